"""The FP64 reference solve (oracle/fp64_mgpcg.py) the accuracy figures are stated against:
it must solve the pressure systems the oracle assembles to FP64 precision, and the oracle's
own FP32 solution (the reference's arithmetic) must sit within the solver tolerance's reach
of it."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.fp64_mgpcg import FP64MGPCG, accuracy
from tests.tanks import dam_break, full_physics


@pytest.fixture(scope="module")
def dam_system():
    t = dam_break(128, 72)
    sim = O.build_tank(t, 4)[0]
    sim.step(3, 3 / 240)
    return t, sim


def test_fp64_solve_reaches_1e_12(dam_system):
    t, sim = dam_system
    s = FP64MGPCG(sim.field("mga"), sim.field("mgd"), t.w, t.h)
    b = sim.field("prhs").astype(np.float64).reshape(t.h, t.w, 4)[..., :2]
    x, rel = s.solve(b)
    assert np.all(rel < 1e-11)
    # and it is the solution: the residual recomputed independently
    assert np.all(s.residual(x, b) < 1e-11)


def test_fp32_solution_is_close_to_fp64(dam_system):
    t, sim = dam_system
    acc = accuracy(sim.field("mga"), sim.field("mgd"), sim.field("prhs"), sim.field("pres"), t.w, t.h)
    # pressure solved to |r| <= 1e-5 |b| in FP32: the error against FP64 is of that order
    assert acc[0]["error_vs_fp64"] < 1e-4
    assert acc[0]["residual_fp64"] < 1e-4


def test_second_solve_system():
    """After a substep with the implicit viscosity the last system is the second solve's
    (b = -div u + A P1, solution P = P1 + P2): its pressure column is checked the same way."""
    t = full_physics(160, 96, cell=0.0064)
    sim = O.build_tank(t, 4)[0]
    sim.step(2, 2 / 240)
    acc = accuracy(sim.field("mga"), sim.field("mgd"), sim.field("prhs"), sim.field("pres"), t.w, t.h, columns=(0,))
    assert acc[0]["fp64_residual"] < 1e-11
    assert acc[0]["error_vs_fp64"] < 1e-2
