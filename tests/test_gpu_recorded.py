"""FluidSim's recorded iteration counts on the device (sprout_sim_recorded_iters) against the
oracle's and against the reference's rule itself. A new scene records pressure_max_iters and
viscosity_max_iters (mod.rs:2478-2483); a solve that has not converged stops at its count
rounded up to even (mod.rs:2569, 2603-2606); after each frame (a step call) the counts adapt
from the frame's solves (mod.rs:3100-3114): half again plus two after a frame whose pressure
column (or viscosity solve) ran out, else the frame's most iterations plus the margin's share
(iters_margin, 0.5 for the viscosity solve) plus two, within [2, max]. The engine adapts when
the frame ends, the reference when the frame's read-back arrives."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_parity import compare_state

pytestmark = pytest.mark.gpu

DT = 1.0 / 240.0


def rule(rec, used, unconverged, mx, margin):
    if unconverged > 0:
        return min(rec + rec // 2 + 2, mx)
    v = used + int(np.float32(used) * np.float32(margin)) + 2
    return max(2, min(v, mx))


def limit(rec):
    return (rec + 1) // 2 * 2


def pair(tank):
    sim, _, _ = tank.engine()
    ora, _, _ = tanks.oracle_of(tank)
    from oracle import oracle as O
    O.set_threads(O.threads_available())
    return sim, ora


@pytest.mark.parametrize("pmax", [60, 10])
def test_recorded_counts_follow_the_reference_rule(pmax):
    tank = tanks.full_physics(96, 64, cell=0.0106)
    tank.settings["pressure_max_iters"] = float(pmax)
    sim, ora = pair(tank)
    vmax = int(S.SimParams(tank.settings).get("viscosity_max_iters"))
    rec = sim.recorded_iters()
    assert rec == ora.recorded_iters() == [pmax, pmax, vmax]
    capped = 0
    for n in [1, 1, 2, 1, 3, 1, 1, 1, 2, 1]:
        a0 = sim.stats()
        sim.step(n, n * DT)
        ora.step(n, n * DT)
        a = sim.stats()
        new = sim.recorded_iters()
        assert new == ora.recorded_iters(), f"recorded {new} vs the oracle's {ora.recorded_iters()}"
        assert max(a.pressure_iters) <= limit(rec[0]) and a.pressure2_iters <= limit(rec[1])
        assert a.viscosity_iters <= limit(rec[2])
        if n == 1:   # the frame's most iterations are this substep's
            un = a.pressure_unconverged - a0.pressure_unconverged
            un2 = a.pressure2_unconverged - a0.pressure2_unconverged
            unv = a.viscosity_unconverged - a0.viscosity_unconverged
            capped += un
            want = [rule(rec[0], max(a.pressure_iters), un, pmax, 0.25),
                    rule(rec[1], a.pressure2_iters, un2, pmax, 0.25),
                    rule(rec[2], a.viscosity_iters, unv, vmax, 0.5)]
            assert new == want, f"recorded {new}, the rule gives {want} (from {rec})"
        rec = new
    problems = compare_state(sim, ora, "after the frames")
    assert not problems, "\n".join(problems[:10])
    if pmax == 10:   # a limit below what the solves need: they stop there, unconverged
        assert capped > 0
