"""The pressure solve that allocates nothing (sprout_pressure_solve_static): for callers that
cannot allocate device memory, it keeps all of its scratch in a fixed array inside the library.
Checked through the C ABI against the engine's own solve (the one a substep runs, whose scratch
the engine allocates): the same system, solved twice in a row, must give the same iterations
and, bit for bit, the same potentials. Covered: a small grid, the largest grid the array
holds (512 x 288), a long thin grid (2048 x 72, whose coarse levels shrink in width only and
need more of the array than a square grid of the same size), and a start from non-zero
potentials, which must come back zero wherever a cell is no unknown.

This file is collected last, so a run that stops at the first failure has run everything else.
"""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks

pytestmark = pytest.mark.gpu


def engine_system(tank):
    """The first substep's pressure system of `tank` (a solve from zero pressure) and the
    engine's solution of it, as host arrays."""
    sim, _, _ = tank.engine()
    sim.step(1, 1.0 / 240.0)
    st = sim.stats()
    n = tank.w * tank.h
    mga = np.ascontiguousarray(sim.field("mga").reshape(-1, 4)[:n])
    mgd = np.ascontiguousarray(sim.field("mgd")[:n])
    rhs = np.ascontiguousarray(sim.field("prhs").reshape(-1, 4)[:n, :2])
    want = sim.field("pres").reshape(-1, 2)
    return mga, mgd, rhs, want, list(st.pressure_iters)


def solve_twice(tank, start=None):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for torch")
    mga, mgd, rhs, want, want_iters = engine_system(tank)
    assert np.count_nonzero(mgd) > 1000 and np.abs(want).max() > 0.0
    dev = torch.device("cuda:0")
    A = torch.from_numpy(mga).to(dev)
    D = torch.from_numpy(mgd).to(dev)
    B = torch.from_numpy(rhs).to(dev)
    n = tank.w * tank.h
    tol_p = tank.settings["pressure_tol"]
    tol_psi = 1e-2   # correction_tol at its default
    for call in range(2):
        if start is None:
            x = torch.zeros((n, 2), dtype=torch.float32, device=dev)
        else:
            x = torch.from_numpy(start).to(dev)
        torch.cuda.synchronize()
        iters, res = S.pressure_solve_static(tank.w, tank.h, A.data_ptr(), D.data_ptr(), B.data_ptr(), x.data_ptr(),
                                             tol_p, tol_psi, 60)
        torch.cuda.synchronize()
        got = x.cpu().numpy()
        yield call, got, iters, res, want, want_iters, mgd


def test_static_solve_matches_the_engine_solve():
    tank = tanks.dam_break(96, 64)
    for call, got, iters, res, want, want_iters, _ in solve_twice(tank):
        assert iters == want_iters, f"call {call}: iterations {iters} vs {want_iters}"
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"call {call}: potentials differ"
        assert res <= tank.settings["pressure_tol"]


@pytest.mark.parametrize("w,h", [(512, 288), (2048, 72)])
def test_static_solve_at_the_array_limits(w, h):
    """The largest grid, and a thin grid of the same order whose hierarchy is the longest."""
    tank = tanks.dam_break(w, h, width=0.5, height=0.6)
    for call, got, iters, res, want, want_iters, _ in solve_twice(tank):
        assert iters == want_iters, f"{w}x{h} call {call}: iterations {iters} vs {want_iters}"
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"{w}x{h} call {call}: potentials differ"


def test_static_solve_zeroes_cells_that_are_no_unknown():
    """Starting from non-zero potentials everywhere (the solve from zero is what the engine
    compares against, so only the cells outside the system are checked here): every cell that
    is no unknown, also in 16 x 16 tiles without any unknown, comes back zero."""
    tank = tanks.dam_break(160, 96, width=0.3, height=0.4)
    n = tank.w * tank.h
    start = np.full((n, 2), 3.0, np.float32)
    for call, got, iters, res, want, want_iters, mgd in solve_twice(tank, start):
        off = ~(mgd > 0)
        assert off.sum() > 2000
        assert np.all(got[off] == 0.0), f"call {call}: {np.count_nonzero(got[off])} values left non-zero"
        assert res <= tank.settings["pressure_tol"]


def test_static_solve_refuses_grids_past_its_array():
    for w, h in [(1024, 576), (513, 288), (15, 64), (9217, 16)]:
        with pytest.raises(S.SproutError) as e:
            S.pressure_solve_static(w, h, 1, 1, 1, 1, 1e-5, 1e-2)
        assert e.value.code == -3, (w, h)
