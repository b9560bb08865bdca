"""Settling suspensions on the CPU (settle.comp with grid_prep.comp:69-70, 147 and
particles.comp:331-352): a concentrate with grains moves down into the clear diluent below,
its total amount conserved; mud also thins with shear."""
import numpy as np
import pytest

import tanks

DT = 1.0 / 240.0


def concentrate(parts, mat):
    live = parts[parts["kind"] != 0]
    m = ((live["kind"] & 255).astype(np.int64) - 1) == mat
    s = live["s"][m].astype(np.float64)
    return float(s.sum()), float((s * live["pos"][m, 1]).sum() / s.sum())


@pytest.mark.parametrize("mat,load", [(51, 0.4), (3, 0.5)])
def test_grains_settle_and_the_concentrate_is_conserved(mat, load):
    ora, parts, _ = tanks.oracle_of(tanks.settling(mat=mat))
    n0 = int(((parts["kind"] & 255) == mat + 1).sum())
    ora.step(1, DT)
    total0, h0 = concentrate(ora.particles(), mat)
    assert abs(total0 - n0 * load) <= 1e-3 * n0, "spawned at the row's load"
    for _ in range(40):
        ora.step(1, DT)
    total1, h1 = concentrate(ora.particles(), mat)
    assert abs(total1 - total0) <= 1e-4 * total0, "settling moves concentrate, never makes it"
    assert h1 < h0, "the grains went down"
    ds = ora.field("dsettle").reshape(-1, 2)
    assert ds[:, 0].max() > 0.0 and ds[:, 1].max() > 0.0
