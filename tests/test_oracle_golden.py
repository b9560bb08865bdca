"""Pins the CPU oracle to the reference's own known-answer tests.

The reference holds no golden vectors for the solver; its unit tests pin the CPU pieces
that build a tank, and those are restated here against the oracle:
  src/scene.rs tests (the_tank_frame_is_solid_and_the_inside_open, open_fraction_follows_the_
  crossing, every_region_has_one_vent_at_its_top, cracks_between_touching_shapes_are_filled,
  shape_distances_have_the_right_sign), src/maps.rs tests (fills_are_rest_density_and_stay_
  inside_the_walls, maps_are_deterministic_and_scale_with_the_grid), and the grid-unit
  conversions of src/sim/params.rs tests (grid_units_follow_the_cell_size).
"""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_lib):
    return oracle_lib


def solid_at(solid, w, i, j):
    return solid[j * w + i]


def test_tank_frame_is_solid_and_inside_open():
    # scene.rs:640-653
    sdf, solid, region, temp = O.rasterize(64, 64)
    assert solid_at(solid, 64, 1, 30)[3] == 0.0
    assert solid_at(solid, 64, 30, 62)[3] == 0.0
    assert solid_at(solid, 64, 3, 30)[0] == 0.0, "the face on the wall is closed"
    assert solid_at(solid, 64, 30, 3)[1] == 0.0, "the face on the floor is closed"
    assert list(solid_at(solid, 64, 30, 30)) == [1.0, 1.0, 0.0, 1.0]
    assert len(sdf) == 65 * 65
    assert temp is None


def test_shape_distances_have_the_right_sign():
    # scene.rs:521-541 (circle and box cases)
    circle = [{"kind": "circle", "c": [10.0, 10.0], "r": 4.0}]
    assert abs(O.lib().oscene_sdf(64, 64, 1, O.shapes_array(circle)[0], 10.0, 10.0) + 4.0) < 1e-5
    assert abs(O.lib().oscene_sdf(64, 64, 1, O.shapes_array(circle)[0], 16.0, 10.0) - 2.0) < 1e-5
    plank = [{"kind": "box", "c": [32.0, 32.0], "half": [10.0, 1.0], "angle": np.pi / 2}]
    arr = O.shapes_array(plank)[0]
    assert O.lib().oscene_sdf(64, 64, 1, arr, 32.0, 41.0) < 0.0, "a quarter turn stands the plank upright"
    assert O.lib().oscene_sdf(64, 64, 1, arr, 41.0, 32.0) > 0.0


def test_open_fraction_via_cut_faces():
    # open_fraction (scene.rs:177-189, tested at scene.rs:587-594): slivers below 5 % close;
    # a face between two fully open cells is open 1.0; every open face leads between open cells.
    shapes = [{"kind": "circle", "c": [128.0, 40.0], "r": 18.0},
              {"kind": "box", "c": [60.0, 30.0], "half": [25.0, 6.0], "angle": 0.5}]
    sdf, solid, region, temp = O.rasterize(256, 144, shapes)
    w, h = 256, 144
    cut = 0
    for j in range(1, h):
        for i in range(1, w):
            left, bottom, occ, op = solid[j * w + i]
            assert 0.0 <= left <= 1.0 and 0.0 <= bottom <= 1.0
            assert op == 0.0 or op >= 0.1
            assert left == 0.0 or left >= 0.05
            if left > 0.0:
                assert op > 0.0 and solid[j * w + i - 1][3] > 0.0
            if bottom > 0.0:
                assert op > 0.0 and solid[(j - 1) * w + i][3] > 0.0
            cut += 0.0 < op < 1.0
    assert cut > 100


def test_every_region_has_one_vent_at_its_top():
    # scene.rs:619-638: a sealed box drawn in the tank is a region of its own
    shapes = [{"kind": "box", "c": c, "half": hf} for c, hf in
              [([64.0, 40.0], [30.0, 2.0]), ([64.0, 80.0], [30.0, 2.0]), ([36.0, 60.0], [2.0, 22.0]), ([92.0, 60.0], [2.0, 22.0])]]
    sdf, solid, region, temp = O.rasterize(128, 128, shapes)
    rid = lambda i, j: region[j * 128 + i] & 31
    assert rid(64, 60) != rid(64, 100)
    assert rid(10, 10) == rid(64, 100)
    assert solid[60 * 128 + 64][3] == 1.0, "the inside of a sealed box stays open"
    for target in (rid(64, 60), rid(64, 100)):
        cells = [k for k in range(128 * 128) if solid[k][3] > 0.0 and (region[k] & 31) == target]
        vents = [k for k in cells if region[k] & 256]
        assert len(vents) == 1
        assert vents[0] // 128 == max(k // 128 for k in cells)
    assert all(s[3] > 0.0 or (r & 256) == 0 for r, s in zip(region, solid))


def test_fills_are_rest_density_and_stay_inside_the_walls():
    # maps.rs:553-563: 64 x 64 tank, rect [0, 0, 64, 23] of honey: 58 x 20 x PPC particles
    out = O.fill_rect(64, 64, [0.0, 0.0, 64.0, 23.0], 1)
    assert len(out) == 58 * 20 * 4
    assert np.all(out["s"] == -1.0)
    assert np.all((out["pos"][:, 0] > 3.0) & (out["pos"][:, 0] < 61.0) & (out["pos"][:, 1] > 3.0))


def test_fills_are_deterministic_and_scale_with_the_grid():
    # maps.rs:538-550 (for one rectangle): the same inputs place the same particles, and
    # twice the resolution holds about four times as many
    a = O.fill_rect(512, 288, [0.0, 0.0, 0.4 * 512, 0.6 * 288], 0)
    b = O.fill_rect(512, 288, [0.0, 0.0, 0.4 * 512, 0.6 * 288], 0)
    assert np.array_equal(a["pos"], b["pos"])
    fine = O.fill_rect(1024, 576, [0.0, 0.0, 0.4 * 1024, 0.6 * 576], 0)
    assert abs(len(fine) / len(a) - 4.0) < 0.2


def test_first_configuration_particle_count():
    # 384 x 216, water over [0, 0, 0.4 W, 0.6 H]: the geometry gives 76,153 particles
    out = O.fill_rect(384, 216, [0.0, 0.0, 0.4 * 384, 0.6 * 216], 0)
    assert len(out) == 76153


def test_oracle_exp_matches_the_true_exponential():
    xs = np.concatenate([np.linspace(-80, 80, 20001, dtype=np.float32), np.float32([-1e-6, 0.0, 1e-6, 0.5, -0.5])])
    got = np.array([O.lib().o_expf(float(x)) for x in xs], np.float64)
    want = np.exp(xs.astype(np.float64))
    rel = np.abs(got - want) / want
    assert rel.max() < 3.6e-7, rel.max()   # within 3 ulp of float32


def test_grid_units_follow_the_cell_size():
    # params.rs:1422-1436: at 1 cm cells gravity is 981 cells/s^2; at 1 mm, 9810
    t = O.default_params()
    assert abs(t.gravity / t.cell_size - 981.0) < 1e-2
    t.cell_size = 0.001
    assert abs(t.gravity / t.cell_size - 9810.0) < 0.1
