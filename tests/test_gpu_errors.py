"""The error paths of the persistent solvers, made on purpose without faulting the GPU.

A grid barrier's wait is bounded. Here one block is made to arrive late (its delay is
measured on the device clock and bounded too) while every block's wait is cut to a few
thousand polls: the waits run out, every block returns, the host reads SPROUT_E_TIMEOUT, and
the context stays usable: after a reset the same sim steps again bit for bit as the oracle.
"""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_parity import compare_state

pytestmark = pytest.mark.gpu

DT = 1.0 / 240.0


def test_late_block_makes_the_barrier_wait_run_out():
    t = tanks.dam_break(160, 96)
    sim, parts, _ = t.engine()
    sim.step_blocking(1)
    assert sim.stats().device_error == 0
    # block 5 of the pressure solve arrives 50 ms late; the others give up after 2000 polls
    sim.debug_stall(5, 50_000_000, 2000)
    with pytest.raises(S.SproutError) as e:
        sim.step_blocking(1)
    assert e.value.code == -5
    assert sim.stats().device_error != 0
    # later solves do nothing until a reset, and report the same
    with pytest.raises(S.SproutError) as e:
        sim.step_blocking(1)
    assert e.value.code == -5
    # a reset clears the error and the injection; the sim then matches the oracle again
    sim.reset(parts)
    ora, _, _ = tanks.oracle_of(t)
    for _ in range(3):
        sim.step(1, DT)
        ora.step(1, DT)
    problems = compare_state(sim, ora, "after the reset")
    assert not problems, "\n".join(problems)
    assert sim.stats().device_error == 0


def test_viscosity_solve_wait_runs_out_too():
    """The same in a tank whose substep also runs the implicit viscosity solve: every
    persistent kernel of the substep returns once the error is set."""
    t = tanks.stratified(128, 72)
    sim, parts, _ = t.engine()
    sim.step_blocking(1)
    assert sim.stats().viscosity_mode == 2
    sim.debug_stall(2, 50_000_000, 2000)
    with pytest.raises(S.SproutError) as e:
        sim.step_blocking(2)
    assert e.value.code == -5
    sim.reset(parts)
    sim.step_blocking(2)
    st = sim.stats()
    assert st.device_error == 0 and st.viscosity_iters_max > 0


def test_non_finite_system_reports_diverged():
    """A pressure system whose right-hand side holds a NaN stops at the solve's start and is
    reported as SPROUT_E_DIVERGED (the reference would count an unconverged solve)."""
    torch = pytest.importorskip("torch")
    t = tanks.dam_break(96, 64)
    sim, _, _ = t.engine()
    sim.step(1, DT)
    n = t.w * t.h
    mga = np.ascontiguousarray(sim.field("mga").reshape(-1, 4)[:n])
    mgd = np.ascontiguousarray(sim.field("mgd")[:n])
    rhs = np.ascontiguousarray(sim.field("prhs").reshape(-1, 4)[:n, :2])
    k = int(np.flatnonzero(mgd > 0)[100])
    rhs[k, 0] = np.nan
    dev = torch.device("cuda:0")
    A, D, B = (torch.from_numpy(a).to(dev) for a in (mga, mgd, rhs))
    x = torch.zeros((n, 2), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    with pytest.raises(S.SproutError) as e:
        S.pressure_solve_static(t.w, t.h, A.data_ptr(), D.data_ptr(), B.data_ptr(), x.data_ptr(), 1e-5, 1e-2, 60)
    assert e.value.code == -4
