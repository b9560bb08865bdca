"""Viscoelastic liquids on the CPU (particles.comp:152-156, 250-279, 983-984, 1053-1058;
grid_prep.comp:241-244; elastic.comp): the particles of slime or putty carry an
upper-convected Maxwell stress that the grid receives and turns into force, capped at
elastic_stress_max x G, and the tank's step limit includes the elastic wave limit."""
import numpy as np
import pytest

import tanks

DT = 1.0 / 240.0


@pytest.mark.parametrize("mat", [12, 33])
def test_stress_reaches_the_grid(mat):
    ora, parts, _ = tanks.oracle_of(tanks.elastic_drop(mat=mat))
    assert ora.stats().caps & 32, "CAP_ELASTIC"
    for _ in range(30):
        ora.step(1, DT)
    e = ora.field("estr").reshape(-1, 4)
    assert np.abs(e[:, :3]).max() > 0.0 and np.all(e[:, 3] == 0.0)
    p = ora.particles()
    assert np.isfinite(p["pos"]).all() and np.isfinite(p["vel"]).all()


def test_elastic_step_limit():
    """Without a fixed rate the substep stays within half a cell of elastic wave travel:
    0.5 dx / sqrt((1 + elastic_stress_max) G / rho) (params.rs:947-960)."""
    import sprout_gb300 as S
    t = tanks.elastic_drop(mat=12)
    t.settings["fixed_hz"] = 0.0
    p = S.SimParams({"cell_size": 0.002})
    limit = 0.5 * 0.002 / np.sqrt(11.0 * 100.0 / p.get("density_slime"))
    ora, _, _ = tanks.oracle_of(t)
    for _ in range(3):
        ora.step(1, 0.0)
    assert 0.0 < ora.stats().dt <= limit * (1 + 1e-6)
