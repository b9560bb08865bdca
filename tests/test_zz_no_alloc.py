"""The pressure solve that allocates nothing (sprout_pressure_solve_static): for callers that
cannot allocate device memory, it keeps all of its scratch in a fixed array inside the library.
Checked through the C ABI against the engine's own solve (the one a substep runs, whose scratch
the engine allocates): the same system, solved twice in a row, must give the same iterations
and, bit for bit, the same potentials.

This file is collected last, so a run that stops at the first failure has run everything else.
"""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks

pytestmark = pytest.mark.gpu


def test_static_solve_matches_the_engine_solve():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for torch")
    tank = tanks.dam_break(96, 64)
    sim, _, _ = tank.engine()
    # The first substep after a reset starts its solve from zero pressure.
    sim.step(1, 1.0 / 240.0)
    st = sim.stats()
    w, h = tank.w, tank.h
    n = w * h
    mga = np.ascontiguousarray(sim.field("mga").reshape(-1, 4)[:n])
    mgd = np.ascontiguousarray(sim.field("mgd")[:n])
    rhs = np.ascontiguousarray(sim.field("prhs").reshape(-1, 4)[:n, :2])
    want = sim.field("pres").reshape(-1, 2)
    assert np.count_nonzero(mgd) > 1000 and np.abs(want).max() > 0.0
    dev = torch.device("cuda:0")
    A = torch.from_numpy(mga).to(dev)
    D = torch.from_numpy(mgd).to(dev)
    B = torch.from_numpy(rhs).to(dev)
    tol_p = tank.settings["pressure_tol"]
    tol_psi = 1e-2   # correction_tol at its default
    for call in range(2):
        x = torch.zeros((n, 2), dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        iters, res = S.pressure_solve_static(w, h, A.data_ptr(), D.data_ptr(), B.data_ptr(), x.data_ptr(), tol_p, tol_psi, 60)
        torch.cuda.synchronize()
        got = x.cpu().numpy()
        assert iters == list(st.pressure_iters), f"call {call}: iterations {iters} vs {list(st.pressure_iters)}"
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"call {call}: potentials differ"
        assert res <= tol_p


def test_static_solve_refuses_grids_past_its_array():
    with pytest.raises(S.SproutError) as e:
        S.pressure_solve_static(1024, 576, 1, 1, 1, 1, 1e-5, 1e-2)
    assert e.value.code == -3
