"""The optics table of the render-side passes (optics.cpp, material.rs optics_table) against
its CPU restatement (oracle/optics.py), bit for bit, for every built-in liquid and for custom
rows that reach every branch (fine particles of both shapes, metal, specks, thermochromic
colour, light of its own, an oily and a freezing melt, a concentrate). Needs the built
library, not a GPU."""
import numpy as np
import pytest

S = pytest.importorskip("sprout_gb300")
from oracle import optics as O

CUSTOM = {
    59: {"cloud": 0.035, "cloud_size": 3e-6, "cloud_ior": 1.46, "ior": 1.35, "opacity": 0.7},   # milk-like
    60: {"metal": 0.9, "gloss": 0.95, "density": 13500.0, "tension": 0.48, "contact_angle": 140.0},
    61: {"dust": 0.05, "dust_size": 3e-4, "dust_shape": 0.3, "dust_reflect": 0.5, "cloud": 0.01, "cloud_shape": 0.2},
    62: {"thermo_lo": 20.0, "thermo_hi": 60.0, "luminous": 1.5, "glow_shear": 0.5, "viscosity": 0.02},
    63: {"melt_lo": 700.0, "melt_hi": 1100.0, "boil": 1e9, "volatility": 0.0, "solids": 0.2, "emissivity": 0.95},
    64: {"volatility": 0.8, "boil": 1e9, "tension": 0.02, "ior": 1.5, "cloud": 0.2, "cloud_ior": 1.6, "cloud_size": 5e-8},
}
COLOURS = {59: {"color": (0.95, 0.95, 0.9)}, 60: {"color": (0.8, 0.8, 0.82), "color_hot": (1.0, 0.5, 0.2)},
           61: {"dust_color": (0.3, 0.25, 0.2), "cloud_color": (0.7, 0.6, 0.5)},
           62: {"color_hot": (0.9, 0.2, 0.6), "glow_color": (0.2, 1.0, 0.3)},
           63: {"color_solid": (0.2, 0.2, 0.2), "color": (1.0, 0.4, 0.05)}}


def params():
    settings = {}
    for row, props in CUSTOM.items():
        for k, v in props.items():
            settings[f"mat{row}.{k}"] = v
    p = S.SimParams(settings)
    for row, cols in COLOURS.items():
        for f, rgb in cols.items():
            assert p.set_color(row, f, rgb)
    assert p.set_group(64, 1) and p.set_group(63, 3)
    assert p.set_diluent(62, 0)
    return p


@pytest.mark.parametrize("custom", [False, True])
def test_optics_table_matches_the_restatement(custom):
    p = params() if custom else S.SimParams()
    rows = range(59, 65) if custom else range(59)
    table = p.optics_table()
    cell, amb, dry, g = p.get("cell_size"), p.get("ambient_temp"), p.get("drying"), p.get("gravity")
    pair0 = [0.0, p.get("tension_oil_water"), p.get("tension_metal_water"), p.get("tension_melt_water")]
    bad = []
    for r in rows:
        want = O.optics_row(p, r, np.float32(cell), np.float32(amb), np.float32(dry), np.float32(g), [np.float32(v) for v in pair0])
        for f in S.OPTICS_FIELDS:
            got = table[r][f]
            w = np.array(want[f], dtype=got.dtype)
            if not np.array_equal(got.view(np.uint32), w.view(np.uint32)):
                bad.append((r, f, got, w))
    assert not bad, bad[:6]


def test_table_is_what_the_reference_describes():
    """Known shapes of the table: water is clear and tints over ~30 cells, milk scatters
    (reduced scattering 1-6 per mm, material.rs's own milk test) with a blue-leaning ratio of
    fine particles; a metal's absorption and scattering follow its colour; a freezing melt
    has a crust; a thermochromic liquid keeps its hot coefficients apart."""
    p = params()
    t = p.optics_table()
    assert t[0]["solid"][3] == pytest.approx(30.5) and t[0]["opt"][0] == 0.0
    cell = p.get("cell_size")
    assert 1.0 < t[59]["absorb"][3] / (cell * 1e3) * 3 < 30.0   # mean reduced scattering per mm, order of milk
    assert t[60]["absorb"][3] > 1.0 and t[60]["opt"][2] == pytest.approx(0.9)
    assert t[63]["fx"][3] > 0.0 and t[63]["idx"][1] == 3
    assert not np.array_equal(t[62]["hot"], t[62]["absorb"])


def test_own_sin_cos_and_atan_within_an_ulp():
    """The ferrofluid spikes' phase takes the engine's own sin, cos and atan (GLSL leaves their
    precision to the implementation; the oracle runs the same FP64 operations, rounded once):
    within an ulp of float64's over the phases and directions the spikes meet."""
    import math
    from oracle import oracle as O
    L = O.lib()
    rng = np.random.default_rng(11)
    for a in np.float32(np.concatenate([rng.uniform(-3000.0, 3000.0, 3000), rng.uniform(-4.0, 4.0, 2000),
                                        [0.0, 1e-30, math.pi, -math.pi / 2, 1e6]])):
        for fn, ref in ((L.o_sinf, math.sin), (L.o_cosf, math.cos)):
            want = ref(float(a))
            got = fn(float(a))
            assert abs(got - want) <= abs(np.spacing(np.float32(want))) + 1e-38, (fn.__name__, a, got, want)
    for y, x in np.float32(rng.uniform(-50.0, 50.0, (4000, 2))).tolist() + [[0.0, 1.0], [1.0, 0.0], [-1.0, -1e-20],
                                                                         [1e-20, -1.0], [3.0, 3.0]]:
        want = math.atan2(float(np.float32(y)), float(np.float32(x)))
        got = L.o_atan2(float(y), float(x))
        assert abs(got - want) <= abs(np.spacing(np.float32(want))) + 1e-38, (y, x, got, want)
    assert L.o_atan2(0.0, 0.0) == 0.0
