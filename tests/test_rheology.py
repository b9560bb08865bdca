"""Non-Newtonian liquids on the CPU: the oracle's ln / pow (the same operations the engine's
device code uses) against float64 within their error bound, and rheo.comp's shear-thinning
viscosity (Carreau, common.glsl:546-571): never above the zero-shear viscosity, lower where the
liquid shears, and the tanks that need rigid bodies still refused."""
import ctypes as C

import numpy as np
import pytest

import tanks

DT = 1.0 / 240.0


def oracle_fn(name, nargs):
    from oracle import oracle as O
    f = getattr(O.lib(), name)
    f.restype = C.c_float
    f.argtypes = [C.c_float] * nargs
    return f


def test_own_log_and_pow_within_their_error_bound():
    logf, powf = oracle_fn("o_logf", 1), oracle_fn("o_powf", 2)
    rng = np.random.default_rng(5)
    xs = np.float32(np.concatenate([np.exp(rng.uniform(-80.0, 80.0, 4000)), [1e-40, 1.0, 2.0, 0.5, 1.4142135, 3.4e38]]))
    for x in xs:
        want = np.log(np.float64(x))
        got = float(logf(float(x)))
        assert abs(got - want) <= 2.5 * abs(np.spacing(np.float32(want))) + 1e-45, (x, got, want)
    for x, y in zip(np.float32(np.exp(rng.uniform(0.0, 20.0, 3000))), np.float32(rng.uniform(-1.5, 0.5, 3000))):
        want = np.float64(x) ** np.float64(y)
        got = float(powf(float(x), float(y)))
        # exp amplifies ln's absolute error by |y ln x| (up to 30 here): a relative bound
        assert abs(got - want) <= (4.0 + 2.0 * abs(y * np.log(x))) * abs(np.spacing(np.float32(want))), (x, y, got, want)
    assert float(powf(1.0, 7.0)) == 1.0 and float(logf(1.0)) == 0.0


@pytest.mark.parametrize("mat", [7, 19])
def test_shear_thinning_viscosity(mat):
    ora, parts, _ = tanks.oracle_of(tanks.shear_thinning(mat=mat))
    from oracle import oracle as O
    for _ in range(12):
        ora.step(1, DT)
    rh, cell = ora.field("rh").reshape(-1, 4), ora.field("cell").reshape(-1, 4)
    mine = (rh[:, 0] > 0.99) & (cell[:, 3] > 0.0)
    assert mine.sum() > 500
    # zero-shear kinematic viscosity in cells^2/s; cell.z = rho x nu
    p = O.default_params()
    nu0 = p.mat[mat].viscosity / 0.002 ** 2
    nu = cell[mine, 2] / cell[mine, 1]
    assert np.all(nu <= nu0 * (1 + 1e-5)), "shear thinning never thickens"
    assert nu.min() < 0.9 * nu0, "sheared cells thinned"
    assert np.all(rh[mine, 1] == mat)


def test_reacting_liquids_stay_refused():
    """Part A and Part B react (the reactions pass is not carried): the oracle refuses the tank,
    as the engine does."""
    t = tanks.shear_thinning(mat=7)
    t.fills = [(t.fills[0][0], 52, None), (t.fills[1][0], 53, None)]
    t.settings = {k: v for k, v in t.settings.items() if not k.startswith("tension_")}
    with pytest.raises(RuntimeError):
        tanks.oracle_of(t)
