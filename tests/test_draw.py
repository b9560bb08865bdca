"""The oracle's restatement of the renderer's particle fields (oracle/draw.py) on its own:
render.rs's test of the wide field's layout, and the plain facts of the passes the engine's
kernels are checked against (tests/test_gpu_draw.py)."""
import numpy as np

import sprout_gb300 as S
from oracle import draw as D

f32 = np.float32


def test_wide_field_fits_its_image_at_every_zoom():
    """render.rs tests::wide_field_fits_its_image_at_every_zoom, on the restated layout."""
    for extent in ([1280, 720], [1920, 1080], [641, 479], [1, 1]):
        for zoom in (0.05, 0.5, 1.5, 2.5, 3.1, 8.0, 25.0, 60.0, 400.0, 1e4):
            w = D.layout((0.0, 0.0), zoom, extent)["wide"]
            image = w["image"]
            assert 1 <= w["w"] <= image[0] and 1 <= w["h"] <= image[1], w
            div = float(w["wide_factor"]) / float(w["factor"])
            assert w["taps"] * 2.0 * div >= float(w["wide_factor"]) * (1 - 1e-6), w
            if D.WIDE_MIN_FACTOR < w["wide_factor"] < D.WIDE_MAX_FACTOR:
                assert abs(float(w["step"]) * 2.0 - float(D.WIDE_SIGMA_TEXELS)) < 1e-3, w


def test_layout_of_a_view():
    """The numbers render.rs computes for a 384 x 256 view at 4 pixels per cell, and far out at
    0.5 (the kernel widened to 1.5 texels, its weight lowered to keep its total)."""
    lay = D.layout((48.0, 32.0), 4.0, (384, 256))
    s, t, w = lay["sharp"], lay["tint"], lay["wide"]
    assert (s["w"], s["h"], float(s["div"]), float(s["radius"]), float(s["weight"])) == (192, 128, 2.0, 1.5, 1.0)
    assert (t["w"], t["h"], float(t["div"])) == (96, 64, 4.0)
    assert (w["w"], w["h"], w["taps"]) == (144, 96, 1) and abs(float(w["step"]) - 1.5) < 1e-6
    far = D.layout((48.0, 32.0), 0.5, (384, 256))["sharp"]
    assert float(far["div"]) == 1.0 and float(far["radius"]) == 3.0 and float(far["weight"]) == 0.25


def particles(rows):
    p = np.zeros(len(rows), S.PARTICLE_DTYPE)
    for k, (pos, vel, row, s) in enumerate(rows):
        p[k]["pos"], p[k]["vel"], p[k]["kind"], p[k]["s"] = pos, vel, row + 1, s
    return p


def test_lone_particle_kernel():
    """A particle at rest: its group's channel peaks at the weight where the kernel is 1 and
    holds weight x pi / 3 x the kernel's radius squared in texels in all; other channels 0."""
    lay = D.layout((20.0, 20.0), 4.0, (160, 160))
    v = lay["sharp"]
    # texel (40, 40)'s centre: x = 20 + (40.5 x 2 - 80) / 4, y = 20 - (40.5 x 2 - 80) / 4 (div 2, zoom 4)
    p = particles([((20.25, 19.75), (0.0, 0.0), 3, 0.0)])
    groups = [0] * 96
    groups[3] = 2
    acc = D.splat(p, groups, np.zeros(96, S.OPTICS_DTYPE), v)
    img = D.unfix(acc).astype(np.float32)
    assert img[..., [0, 1, 3]].max() == 0.0
    assert abs(img[..., 2].max() - 1.0) < 1e-3
    r_tex = float(v["radius"]) * 4.0 / 2.0
    assert abs(img[..., 2].sum() - np.pi / 3.0 * r_tex * r_tex) < 0.05 * np.pi / 3.0 * r_tex * r_tex


def test_streak_keeps_its_front_on_the_particle():
    """A fast particle is drawn stretched back along its path: the kernel reaches a radius ahead
    of it and a radius + the streak behind, the streak at most 1.5 radii."""
    lay = D.layout((30.0, 20.0), 4.0, (240, 160))
    v = lay["sharp"]
    groups = [0] * 96
    p = particles([((30.0, 20.0), (400.0, 0.0), 0, 0.0)])   # 2.5 cells in 1/160 s: the cap
    img = D.unfix(D.splat(p, groups, np.zeros(96, S.OPTICS_DTYPE), v)).astype(np.float32)[..., 0]
    cols = np.nonzero(img.sum(axis=0) > 0)[0]
    x_lo = 30.0 + ((cols.min() + 0.5) * 2.0 - 120.0) / 4.0   # texel centre -> cells (div 2, zoom 4)
    x_hi = 30.0 + ((cols.max() + 0.5) * 2.0 - 120.0) / 4.0
    front, back = x_hi - 30.0, 30.0 - x_lo
    assert 1.5 - 0.5 <= front <= 1.5 and back >= 1.5 + 2.25 - 0.5
    assert back <= 1.5 + 2.25


def test_tint_payload():
    """The tint field: an aqueous concentrate at s lays its absorption times s and its
    scattering blended with the diluent's; the share image (s, 1, 0); another group (0, 0, 1)."""
    optics = np.zeros(96, S.OPTICS_DTYPE)
    optics[1]["absorb"] = (0.2, 0.4, 0.8, 1.0)
    optics[1]["idx"] = (0, 0, 0, 0)
    optics[0]["absorb"] = (0.0, 0.0, 0.0, 3.0)
    optics[0]["idx"] = (-1, 0, 0, 0)
    optics[2]["absorb"] = (0.5, 0.5, 0.5, 0.5)
    optics[2]["idx"] = (-1, 1, 0, 0)
    groups = [0] * 96
    groups[2] = 1
    v = D.layout((20.0, 20.0), 4.0, (160, 160))["tint"]
    for row, s, want, share in ((1, 0.25, (0.05, 0.1, 0.2, 0.25 + 0.75 * 3.0), (0.25, 1.0, 0.0)),
                                (2, 0.0, (0.5, 0.5, 0.5, 0.5), (0.0, 0.0, 1.0))):
        p = particles([((20.5, 19.5), (0.0, 0.0), row, s)])   # a texel centre (div 4, zoom 4)
        img = D.unfix(D.splat(p, groups, optics, v)).astype(np.float32)
        peak = np.unravel_index(np.argmax(img[..., 5] + img[..., 6]), img.shape[:2])
        np.testing.assert_allclose(img[peak][:4], want, rtol=2e-3)
        np.testing.assert_allclose(img[peak][4:7], share, rtol=2e-3, atol=1e-3)


def test_filters_keep_a_constant_field():
    """down.frag and blur.frag average: a uniform field passes unchanged (to the half float)."""
    img = np.full((40, 60, 4), 0.7, np.float16)
    lay = D.layout((0.0, 0.0), 6.0, (120, 80))
    w = lay["wide"]
    d = D.down(img, w)
    assert d.shape == (w["h"], w["w"], 4)
    assert np.all(d == np.float16(0.7))
    b = D.blur(d, w["step"], vert=False)
    assert np.all(np.abs(b.astype(np.float32) - 0.7) <= 1e-3)


def test_wet_map_rules():
    """A cell within 1.75 cells of a solid holding liquid (occupancy >= 0.3) records its leading
    material row + 1 (the fraction of its group code), family 0's concentration and the time;
    the rest keep what they had."""
    H, W = 3, 4
    sdf = np.full((H + 1, W + 1), 5.0, np.float32)
    sdf[:, 0], sdf[:, 1] = 0.0, 1.0   # a wall along the left: cells x = 0 lie against it (mean 0.5)
    cell = np.zeros((H, W, 4), np.float32)
    cell[..., 0] = 1.0
    cell[2, 0, 0] = 0.1   # too little liquid
    comp = np.zeros((H, W, 4), np.float32)
    comp[..., 2] = 0.5
    sprop = np.zeros((H, W, 4), np.float32)
    sprop[..., 3] = 1.0 + 6.0 / 128.0   # group 1, row 5
    prev = np.zeros((H, W, 4), np.float32)
    prev[2, 0] = (9.0, 0.0, 0.5, 1.0)
    out = D.wet(prev, cell, comp, sdf, sprop, np.float32(2.5))
    assert tuple(out[0, 0]) == (6.0, 0.5, 2.5, 1.0) and tuple(out[1, 0]) == (6.0, 0.5, 2.5, 1.0)
    assert tuple(out[2, 0]) == (9.0, 0.0, 0.5, 1.0)
    assert np.all(out[:, 1:] == 0.0)
