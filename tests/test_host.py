"""Host-side tests of the engine library that need no GPU: it loads and exports every entry
point of include/sprout_gpu.h; its parameter table behaves as SimParams::set does in the
reference's own tests (src/sim/params.rs:1336-1364); its scene rasterisation and particle
fill agree with the oracle bit for bit."""
import math
import re
from pathlib import Path

import numpy as np
import pytest

import sprout_gb300 as S
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]


def f32(x):
    return float(np.float32(x))


@pytest.fixture(scope="module", autouse=True)
def _libs(engine_lib, oracle_lib):
    return engine_lib


def test_library_exports_every_declared_entry_point():
    header = (ROOT / "include" / "sprout_gpu.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|const char\*)\s+(sprout_\w+)\s*\(", header, re.M))
    assert declared == set(S.EXPORTS)
    lib = S.lib()
    for name in declared:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.sprout_version()


def test_overrides_reach_the_named_parameter():
    # params.rs:1336-1364
    p = S.SimParams()
    assert p.set("viscosity_honey", 0.09) and p.get("viscosity_honey") == f32(0.09)
    assert p.set("nu_honey", 0.08) and p.get("honey.viscosity") == f32(0.08), "old names still work"
    assert p.set("honey.viscosity", 0.07) and p.get("viscosity_honey") == f32(0.07)
    assert p.set("density_oil", 800.0) and p.get("density_oil") == 800.0
    assert p.set("tension_water", 0.05) and p.get("tension_water") == f32(0.05)
    assert p.set("sigma_water", 0.06) and p.get("tension_water") == f32(0.06)
    assert p.set("contact_angle_oil", 200.0) and p.get("contact_angle_oil") == 180.0, "clamped to the range"
    assert p.set("contact_oil", 30.0) and p.get("contact_angle_oil") == 30.0
    assert p.set("tension_oil_water", 0.03) and p.get("tension_oil_water") == f32(0.03)
    assert p.set("mat40.density", 1234.0) and p.get("density_mat40") == 1234.0, "custom rows by number"
    assert p.set("pressure_iters", 50.4) and p.get("pressure_max_iters") == 50.0
    assert p.set("substep_hz", 1.0) and p.get("fixed_hz") == 30.0, "a fixed rate has a floor"
    assert p.set("fixed_hz", 0.0) and p.get("fixed_hz") == 0.0, "0 selects the adaptive step"
    assert p.set("mix_rate", -5.0) and p.get("mix_rate_honey") == 0.0
    assert p.set("diffuse", 2.0) and p.get("mix_rate_honey") == 2.0
    assert p.set("speed_cap", 0.0) and p.get("speed_cap") == 0.0, "0 switches the cap off"
    g = p.get("gravity")
    assert not p.set("gravity", math.nan) and p.get("gravity") == g, "NaN is refused"
    assert p.set("gravity", math.inf) and math.isfinite(p.get("gravity")), "infinity is clamped"
    assert p.set("speed_cap", 0.3) and p.get("speed_cap") == 1.0
    assert not p.set("no_such_parameter", 1.0)
    assert not p.set("viscosity_unobtainium", 1.0)
    assert not p.set("rho_oil", 0.8), "relative density is gone"
    assert not p.set("rest_phi", 1.0) and not p.set("fluid_thr", 0.5), "definitions, not settings"
    assert not p.set("sigma_oil", 0.03), "ambiguous old name"


def test_parameter_defaults():
    # params.rs:386-451, presets.rs:37-117
    p = S.SimParams()
    assert p.get("cell_size") == pytest.approx(0.01)
    assert p.get("cfl") == 4.0 and p.get("pressure_tol") == pytest.approx(1e-4)
    assert p.get("pressure_max_iters") == 60.0
    assert p.get("viscosity_water") == pytest.approx(1e-6)
    assert p.get("density_honey") == pytest.approx(1.4 * 998.0)
    assert p.get("density_oil") == pytest.approx(0.9 * 998.0)
    assert p.get("tension_oil_water") == pytest.approx(0.025)
    assert p.get("correction_time") == pytest.approx((1 / 240) / math.log(2), rel=1e-6)


SCENES = [
    (64, 64, []),
    (256, 144, [{"kind": "circle", "c": [128.0, 40.0], "r": 18.0},
                {"kind": "box", "c": [60.0, 30.0], "half": [25.0, 6.0], "angle": 0.5}]),
    (128, 128, [{"kind": "box", "c": c, "half": hf} for c, hf in
                [([64.0, 40.0], [30.0, 2.0]), ([64.0, 80.0], [30.0, 2.0]), ([36.0, 60.0], [2.0, 22.0]), ([92.0, 60.0], [2.0, 22.0])]]),
    (192, 108, [{"kind": "box", "c": [96.0, 7.0], "half": [96.0, 4.0], "angle": 0.0, "temp": 326.85}]),
]


def engine_scene(w, h, shapes):
    sc = S.Scene(w, h)
    for s in shapes:
        if s["kind"] == "box":
            sc.add_box(s["c"], s["half"], s.get("angle", 0.0), s.get("temp"))
        else:
            sc.add_circle(s["c"], s["r"], s.get("temp"))
    return sc


@pytest.mark.parametrize("w,h,shapes", SCENES)
def test_scene_rasterize_matches_oracle(w, h, shapes):
    a = engine_scene(w, h, shapes).rasterize()
    b = O.rasterize(w, h, shapes)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert (a[3] is None) == (b[3] is None)
    if a[3] is not None:
        assert np.array_equal(a[3], b[3])


@pytest.mark.parametrize("w,h,shapes", SCENES)
def test_fill_rect_matches_oracle(w, h, shapes):
    rect = [0.0, 0.0, 0.5 * w, 0.7 * h]
    a = engine_scene(w, h, shapes).fill_rect(rect, 0)
    b = O.fill_rect(w, h, rect, 0, shapes)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    # a second rectangle is seeded by the count before it (maps.rs:473)
    a2 = engine_scene(w, h, shapes).fill_rect([0.6 * w, 0.0, w, 0.3 * h], 0, a)
    b2 = O.fill_rect(w, h, [0.6 * w, 0.0, w, 0.3 * h], 0, shapes, b)
    assert np.array_equal(a2.view(np.uint8), b2.view(np.uint8))


def test_scene_sdf_matches_oracle():
    w, h, shapes = SCENES[1]
    sc = engine_scene(w, h, shapes)
    arr, n = O.shapes_array(shapes)
    for x, y in [(10.0, 10.0), (128.0, 40.0), (60.0, 30.0), (1.0, 1.0), (200.5, 100.25)]:
        assert sc.sdf(x, y) == O.lib().oscene_sdf(w, h, n, arr, x, y)


def test_bad_arguments_return_errors():
    p = S.SimParams()
    with pytest.raises(S.SproutError) as e:
        S.FluidSim(8, 8, 100, p)
    assert e.value.code == -1
