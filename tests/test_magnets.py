"""Magnets on the CPU (params.rs:1082-1087, magnet.comp, grid_prep.comp:63, 168, 216-220,
240): a magnetic liquid is drawn up towards a magnet placed above it, and without magnets
(or without a susceptible liquid) magnet.comp does not run."""
import numpy as np
import pytest

import tanks

DT = 1.0 / 240.0


def heights(ora, mat):
    p = ora.particles()
    live = p[p["kind"] != 0]
    y = live["pos"][((live["kind"] & 255).astype(np.int64) - 1) == mat, 1]
    return float(y.mean()), float(y.max())


@pytest.mark.parametrize("mat,demag", [(37, 0.0), (13, 0.5)])
def test_magnet_draws_its_liquid_up(mat, demag):
    pulled, free = [], []
    for with_magnet, out in [(True, pulled), (False, free)]:
        t = tanks.magnetic(mat=mat, demag=demag)
        if not with_magnet:
            t.magnets = []
        ora, _, _ = tanks.oracle_of(t)
        assert bool(ora.stats().caps & 16) == with_magnet
        for _ in range(30):
            ora.step(1, DT)
        out.extend(heights(ora, mat))
    assert pulled[0] > free[0] + 5.0 and pulled[1] > free[1] + 10.0


def test_magnet_records_match_the_reference_layout():
    import sprout_gb300 as S
    assert S.MAGNET_DTYPE.itemsize == 24
    arr = S.magnet_array([{"pos": (1.0, 2.0), "radius": 3.0, "strength": 0.5, "dir": (0.0, -1.0)}])
    assert arr.view(np.float32).tolist() == [1.0, 2.0, 3.0, 0.5, 0.0, -1.0]
