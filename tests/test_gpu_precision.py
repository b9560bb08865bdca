"""The mixed-precision pressure solve (BF16 hierarchy, FP32 iterate and residual, FP64 dot
products and convergence test) against the plain FP32 solve and the FP64 reference solution,
on the same tanks.

Mixed precision changes the preconditioner's rounding, so its results are not bit-exact with
the reference's arithmetic; what must hold is the reference's own stopping rule (the same
relative residual of the carried residual, pressure_tol = 1e-5) and a true residual, evaluated
in FP64, of the same order as the plain solve's. Neither can go below the FP32 floor: the
FP64 solution itself, rounded to FP32, leaves a relative residual of ~5e-5 on a dam break and
~1e-3 on the sealed full-physics pour, so the bounds here are stated against that floor and
against the plain arm on the same system, with the factors written in the tests.
"""
import numpy as np
import pytest

import tanks
from oracle.fp64_mgpcg import FP64MGPCG, accuracy


def fp32_floor(sim, tank) -> float:
    """|b - A fl32(x*)| / |b| of the FP64 solution x* of the last pressure system, rounded to FP32."""
    s = FP64MGPCG(sim.field("mga"), sim.field("mgd"), tank.w, tank.h)
    b = np.asarray(sim.field("prhs"), np.float64).reshape(tank.h, tank.w, 4)[..., :2]
    x, _ = s.solve(b)
    return float(s.residual(x.astype(np.float32).astype(np.float64), b)[0])

pytestmark = pytest.mark.gpu


def pair(tank):
    a, _, _ = tank.engine()
    b, _, _ = tank.engine()
    b.set_precision("mixed")
    return a, b


def last_system_accuracy(sim, tank, columns):
    return accuracy(sim.field("mga"), sim.field("mgd"), sim.field("prhs"), sim.field("pres"), tank.w, tank.h,
                    columns=columns)


def test_mixed_first_solve_matches_plain():
    """The first substep from the same state: both solve the same system (everything before
    the solve is the same FP32 arithmetic), to the same tolerance, and agree with each other
    and with the FP64 solution to the order of that tolerance."""
    t = tanks.dam_break(128, 72)
    plain, mixed = pair(t)
    plain.step(1, 1 / 240.0)
    mixed.step(1, 1 / 240.0)
    for s in (plain, mixed):
        st = s.stats()
        assert st.device_error == 0 and st.pressure_unconverged == 0
    # the same system (prhs.xy; prhs.z keeps each one's own solution for the projection)
    assert np.array_equal(plain.field("prhs").reshape(-1, 4)[:, :2], mixed.field("prhs").reshape(-1, 4)[:, :2])
    pp = plain.field("pres").reshape(-1, 2)[:, 0].astype(np.float64)
    pm = mixed.field("pres").reshape(-1, 2)[:, 0].astype(np.float64)
    assert np.linalg.norm(pm - pp) <= 1e-4 * np.linalg.norm(pp)
    ap = last_system_accuracy(plain, t, (0,))
    am = last_system_accuracy(mixed, t, (0,))
    # stopping rule 1e-5 on the carried residual; against the FP64 solution both within 5e-5,
    # and the FP64 true residual within 4x of the larger of the plain arm's and the FP32 floor
    assert ap[0]["error_vs_fp64"] < 5e-5 and am[0]["error_vs_fp64"] < 5e-5, (ap, am)
    floor = fp32_floor(plain, t)
    assert am[0]["residual_fp64"] <= 4.0 * max(ap[0]["residual_fp64"], floor), (am, ap, floor)
    assert mixed.stats().pressure_residual <= 1e-5 * 1.0001
    # the FP64 true residual the mixed solve reports agrees with the one computed here
    assert abs(mixed.stats().pressure_true_residual - am[0]["residual_fp64"]) <= 1e-3 * am[0]["residual_fp64"] + 1e-9


def test_mixed_keeps_converging_over_a_run():
    t = tanks.dam_break(128, 72)
    plain, mixed = pair(t)
    for s in (plain, mixed):
        s.step(24, 24 / 240.0)
    sp, sm = plain.stats(), mixed.stats()
    assert sm.device_error == 0 and sm.pressure_unconverged == 0
    assert sm.pressure_residual_max <= 1e-5 * 1.0001
    # the BF16 preconditioner is a little weaker: at most half as many iterations again
    assert max(sm.pressure_iters) <= 1.5 * max(sp.pressure_iters) + 2


def test_mixed_runs_the_full_physics_pour():
    t = tanks.full_physics(160, 96, cell=0.0064)
    plain, mixed = pair(t)
    for s in (plain, mixed):
        s.step(12, 12 / 240.0)
    sp, sm = plain.stats(), mixed.stats()
    assert sm.device_error == 0
    assert sm.pressure_unconverged == 0 and sm.pressure2_unconverged == 0
    assert sm.pressure_residual_max <= 1e-5 * 1.0001
    # the tanks evolve alike: particle positions within a small fraction of a cell
    g = np.sort(plain.download_particles(), order="id")
    m = np.sort(mixed.download_particles(), order="id")
    assert np.array_equal(g["id"], m["id"])
    d = np.abs(g["pos"] - m["pos"]).max()
    assert d < 0.05, d
    # the last system of each arm: true residual (FP64) within 4x of the larger of the plain
    # arm's and the FP32 floor, error against the FP64 solution within 4x of the plain arm's
    am = last_system_accuracy(mixed, t, (0,))
    ap = last_system_accuracy(plain, t, (0,))
    floor = max(fp32_floor(mixed, t), fp32_floor(plain, t))
    assert am[0]["residual_fp64"] <= 4.0 * max(ap[0]["residual_fp64"], floor), (am, ap, floor)
    assert am[0]["error_vs_fp64"] <= 4.0 * max(ap[0]["error_vs_fp64"], 1e-5), (am, ap)
    assert abs(sm.pressure_true_residual - am[0]["residual_fp64"]) <= 1e-3 * am[0]["residual_fp64"] + 1e-9


def test_refinement_keeps_the_plain_arms_true_residual():
    """The refinement (residual replacement, checked against the FP32 rounding floor) leaves
    the mixed solve converged to the reference's tolerance, with a true residual within 2x of
    the plain solve's, or of the floor where that is larger: a replacement is adopted only
    well above the floor, so none can have pushed the residual there."""
    t = tanks.dam_break(256, 144)
    plain, mixed = pair(t)
    for s in (plain, mixed):
        s.step(16, 16 / 240.0)
    sm = mixed.stats()
    assert sm.device_error == 0 and sm.pressure_unconverged == 0 and sm.pressure2_unconverged == 0
    assert sm.pressure_residual_max <= 1e-5 * 1.0001
    am = last_system_accuracy(mixed, t, (0,))
    ap = last_system_accuracy(plain, t, (0,))
    floor = fp32_floor(mixed, t)
    assert am[0]["residual_fp64"] <= 2.0 * max(ap[0]["residual_fp64"], floor), (am, ap, floor)
    assert plain.stats().pressure_replacements == 0   # the plain arm is the reference's arithmetic
