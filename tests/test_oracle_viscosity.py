"""The oracle's implicit viscosity (visc_diag.comp, vmg_build.comp, vmg.glsl, visc_mgu.comp,
visc_mgz.comp, reduce_tail.glsl modes 4-13): properties the reference's construction implies.

The reference builds the level-0 matrix of the viscosity multigrid by hand (visc_diag.comp:
couplings) from the same weighted-strain operator its iterations apply matrix-free
(visc_iter.comp). Both must be the same matrix, symmetric, and every coarse level must be the
Galerkin product R A P of the level above (vmg_build.comp). The solve itself must reach the
relative residual it is asked for.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.tanks import stratified

W, H = 128, 72


@pytest.fixture(scope="module")
def viscous_sim():
    sim = O.build_tank(stratified(W, H), 4)[0]
    sim.step(3)
    return sim


def test_stratified_tank_takes_the_implicit_solve(viscous_sim):
    st = viscous_sim.stats()
    assert st.viscosity_mode == 2
    tiles = viscous_sim.field("tiles", np.uint32)
    assert 0 < tiles.sum() < tiles.size          # the honey layer only


def test_assembled_matrix_is_the_strain_operator(viscous_sim):
    x = np.random.default_rng(1).standard_normal(W * H * 2).astype(np.float32)
    n, a, b = viscous_sim.visc_operator(x)
    assert n > 1000
    # the same sums in another order: float32 rounding only
    assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()


@pytest.mark.parametrize("level", [0, 1])
def test_levels_are_symmetric(viscous_sim, level):
    w, h = W >> level, H >> level
    rng = np.random.default_rng(level)
    x = rng.standard_normal(w * h * 2).astype(np.float32)
    y = rng.standard_normal(w * h * 2).astype(np.float32)
    ax = viscous_sim.vmg_apply(level, x).astype(np.float64)
    ay = viscous_sim.vmg_apply(level, y).astype(np.float64)
    lhs, rhs = float(y @ ax), float(x @ ay)
    assert abs(lhs - rhs) <= 1e-6 * (np.abs(y * ax).sum())


def test_coarse_level_is_galerkin_product(viscous_sim):
    w, h = W // 2, H // 2
    xc = np.random.default_rng(7).standard_normal((h, w, 2)).astype(np.float32)
    xf = np.repeat(np.repeat(xc, 2, 0), 2, 1)[:H, :W]
    yf = viscous_sim.vmg_apply(0, xf.reshape(-1)).reshape(H, W, 2)
    yr = yf.reshape(h, 2, w, 2, 2).sum(axis=(1, 3))
    yc = viscous_sim.vmg_apply(1, xc.reshape(-1)).reshape(h, w, 2)
    vmd = viscous_sim.field("vmd")
    dc = vmd[2 * W * H: 2 * (W * H + w * h)].reshape(h, w, 2)
    mask = dc > 0
    assert mask.sum() > 100
    assert np.abs((yc - yr)[mask]).max() <= 1e-5 * np.abs(yc[mask]).max()


def test_solves_reach_their_tolerance(viscous_sim):
    st = viscous_sim.stats()
    assert st.v_unconv == 0 and st.p_unconv == 0 and st.p2_unconv == 0
    assert 0 < st.v_it_max < 50
    assert st.v_res_max <= 1e-5
    assert st.p2_it_max > 0                     # the second projection ran


def test_jacobi_preconditioned_solve_reaches_the_same_velocities():
    """viscosity_precond 0 (visc_iter.comp / visc_update.comp, cg_reduce modes 5 and 6): the
    Jacobi-preconditioned iteration solves the same system to the same tolerance as the
    multigrid one, in more iterations."""
    mg = O.build_tank(stratified(W, H, extra={"viscosity_warm": 0}), 4)[0]
    jac = O.build_tank(stratified(W, H, extra={"viscosity_warm": 0, "viscosity_precond": 0}), 4)[0]
    mg.step(1)
    jac.step(1)
    a, b = mg.stats(), jac.stats()
    assert a.viscosity_mode == b.viscosity_mode == 2
    assert b.v_unconv == 0 and b.v_res_max <= 1e-5 and b.v_it_max > a.v_it_max > 0
    va, vb = mg.field("vel").reshape(-1, 4), jac.field("vel").reshape(-1, 4)
    scale = np.abs(va[:, :2]).max()
    assert np.abs(va[:, :2] - vb[:, :2]).max() <= 1e-4 * scale
