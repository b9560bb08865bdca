"""The renderer's particle fields on the device (sprout_sim_draw: the splat, tint, down and blur
passes of Renderer::render, render.rs:886-1075, and wet.frag's wet map) against the oracle's
restatement (oracle/draw.py) on the engine's own particles and grid, bit for bit in every
texel. Views near and far (the kernel widened below 1.5 texels, the sharp field at full and at
half resolution), tanks with and without two liquids of one phase group (the tint field drawn
or left alone), moving liquid (streaks), the look field of a liquid carrying platelets, and the
wet map kept over frames."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from oracle import draw as D

pytestmark = pytest.mark.gpu


def table_of(tank):
    table = S.SimParams(tank.settings)
    for row, dil in tank.diluents.items():
        table.set_diluent(row, dil)
    for row, grp in tank.groups.items():
        table.set_group(row, grp)
    return table


def oracle_fields(sim, tank, center, zoom, size):
    parts = sim.download_particles()
    table = table_of(tank)
    groups = [table.row_kind(r)[0] for r in range(96)]
    optics = table.optics_table()
    rows = sorted({(int(k) & 255) - 1 for k in parts["kind"] if int(k) & 255})
    live = len(parts) > 0 and D.shares_a_group(rows, groups)
    lay = D.layout(center, zoom, size, live)
    sharp, conc, share = D.fields(parts, groups, optics, lay)
    return lay, sharp, conc, share, D.wide_field(sharp, lay["wide"])


def same(a, b, what):
    assert a is not None and b is not None, what
    assert a.shape == b.shape, f"{what}: {a.shape} vs {b.shape}"
    ua, ub = a.view(np.uint16), b.view(np.uint16)
    bad = np.argwhere(ua != ub)
    assert len(bad) == 0, (f"{what}: {len(bad)} half words differ, first texel {tuple(bad[0][:2][::-1])} channel "
                           f"{bad[0][2]}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}")


@pytest.mark.parametrize("name,zoom,size", [("honey_dam", 4.0, (384, 256)), ("honey_dam", 0.9, (200, 150)),
                                            ("water_oil", 7.5, (320, 200)), ("full_physics", 2.2, (301, 181)),
                                            ("dam_break", 12.0, (640, 360))])
def test_fields_bit_exact(name, zoom, size):
    tank = {"honey_dam": lambda: tanks.honey_dam(), "water_oil": lambda: tanks.water_oil(),
            "full_physics": lambda: tanks.full_physics(96, 64, cell=0.0106),
            "dam_break": lambda: tanks.dam_break(96, 64)}[name]()
    sim, _, _ = tank.engine()
    sim.step(6, 6 / 240.0)
    sim.sync()
    center = (sim.w * 0.5 + 3.25, sim.h * 0.5 - 1.5)
    sim.draw(center, zoom, size)
    lay, sharp, conc, share, wide = oracle_fields(sim, tank, center, zoom, size)
    e_sharp = sim.download_draw("sharp")
    assert e_sharp.shape[:2] == (lay["sharp"]["h"], lay["sharp"]["w"])
    same(e_sharp, sharp, "sharp field")
    same(sim.download_draw("wide"), wide, "wide field")
    if lay["tint"] is None:
        assert sim.download_draw("tint") is None
    else:
        same(sim.download_draw("tint"), conc, "tint field")
        same(sim.download_draw("share"), share, "tint share")
        assert float(share[..., 1].astype(np.float32).max()) > 0.0
    # something was drawn: the liquid's groups reach the surface threshold (0.65) inside it
    assert float(e_sharp.astype(np.float32).sum(axis=2).max()) > 0.65
    assert float(wide.astype(np.float32).max()) > 0.0
    parts = sim.download_particles()
    live = parts[(parts["kind"] & 255) != 0]
    assert float(np.hypot(live["vel"][:, 0], live["vel"][:, 1]).max()) * float(D.EXPOSURE) > 0.01   # streaks


def test_wet_map_over_frames():
    """wet.frag: written where liquid lies against a solid, kept elsewhere, once per simulated
    time; a draw without a substep since leaves it as it was."""
    tank = tanks.dam_break(96, 64)
    sim, _, _ = tank.engine()
    W, H = sim.w, sim.h
    ora = np.zeros((H, W, 4), np.float32)
    for frame in range(3):
        sim.step(4, 4 / 240.0)
        sim.sync()
        sim.draw((W * 0.5, H * 0.5), 3.0, (288, 192))
        f = {n: sim.field(n) for n in ("cell", "comp", "sprop", "sdf")}
        ora = D.wet(ora, f["cell"].reshape(H, W, 4), f["comp"].reshape(H, W, 4), f["sdf"].reshape(H + 1, W + 1),
                    f["sprop"].reshape(H, W, 4), np.float32(sim.stats().sim_time))
        e = sim.download_draw("wet")
        assert np.array_equal(e.view(np.uint32), ora.view(np.uint32)), f"frame {frame}"
    assert (e[..., 3] == 1.0).sum() > 10
    assert len(np.unique(e[e[..., 3] == 1.0][:, 2])) >= 2   # cells last wet in different frames
    sim.draw((W * 0.5, H * 0.5), 3.0, (288, 192))
    assert np.array_equal(sim.download_draw("wet").view(np.uint32), e.view(np.uint32))


def test_draw_rejects_bad_views():
    tank = tanks.dam_break(96, 64)
    sim, _, _ = tank.engine()
    for center, zoom, size in (((10, 10), 0.0, (64, 64)), ((10, 10), float("nan"), (64, 64)),
                               ((10, 10), 2.0, (0, 64)), ((10, 10), 2.0, (64, 20000))):
        with pytest.raises(S.SproutError):
            sim.draw(center, zoom, size)


def test_look_field_bit_exact():
    """look.vert + look.frag over the particles look.comp listed (a dam break of water carrying
    mica platelets): every texel of the look field equals the oracle's from the same state and
    list; a tank without a liquid with a look leaves it clear."""
    mica = {"mat0.cloud": 0.05, "mat0.cloud_shape": 0.05, "mat0.cloud_size": 1.5e-5}
    tank = tanks.dam_break(96, 64, extra=mica)
    sim, _, _ = tank.engine()
    sim.step(6, 6 / 240.0)
    sim.render(1.0 / 80.0)
    for center, zoom, size in (((48.0, 30.0), 4.0, (384, 256)), ((40.5, 20.25), 0.8, (160, 100))):
        sim.draw(center, zoom, size)
        st, lst = sim.download_look()
        lay = D.layout(center, zoom, size)
        want = D.look_field(sim.download_particles(), st, lst, lay)
        same(sim.download_draw("look"), want, f"look field at zoom {zoom}")
        w = want.astype(np.float32)
        assert w[..., 3].max() > 0.5 and w[..., 0].max() > 0.0
    plain = tanks.dam_break(96, 64)
    sim2, _, _ = plain.engine()
    sim2.step(2, 2 / 240.0)
    sim2.render(1.0 / 80.0)
    sim2.draw((48.0, 30.0), 4.0, (384, 256))
    assert not sim2.download_draw("look").astype(np.float32).any()
