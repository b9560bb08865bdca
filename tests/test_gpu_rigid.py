"""Rigid bodies on the GPU, bit for bit against the oracle: the labels and union-find of
rigid.comp (roots do not depend on the order of the atomics), the bodies' 64-bit sums and
contacts, the faces moved with their body, and the particles held by it."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


def test_yield_stress_bodies_bit_exact():
    sim, ora, problems = run_pair(tanks.yield_stress(mat=5), 16)
    assert not problems, "\n".join(problems[:10])
    a, b = sim.field("rl", np.int32).reshape(-1, 2), ora.field("rl", np.int32).reshape(-1, 2)
    assert np.array_equal(a[:, 0], b[:, 0]), "labels"
    assert (a[:, 0] >= 0).any()


def test_rigid_tank_in_a_batch_equals_alone():
    def variants():
        return [tanks.yield_stress(mat=5), tanks.dam_break(96, 64)]
    alone = [t.engine()[0] for t in variants()]
    batched = [t.engine()[0] for t in variants()]
    batch = S.Batch(batched, "plain")
    n = 6
    for s in alone:
        s.step(n, n / 240.0)
    batch.step(n)
    batch.sync()
    problems = []
    for k, (a, b) in enumerate(zip(alone, batched)):
        problems += compare(a, b, f"tank {k}")
    assert not problems, "\n".join(problems)


def test_freezing_lava_bit_exact():
    """Heat and freezing: the frozen share of the cells (therm.w) makes them rigid, and the
    frozen particles move with the body."""
    sim, ora, problems = run_pair(tanks.cooling_lava(), 24)
    assert not problems, "\n".join(problems[:10])
    a, b = sim.field("rl", np.int32).reshape(-1, 2), ora.field("rl", np.int32).reshape(-1, 2)
    assert np.array_equal(a[:, 0], b[:, 0]) and (a[:, 0] >= 0).sum() > 100


def test_clay_combined_capabilities_bit_exact():
    """Clay slip: a water concentrate (family) with grains (settling), a yield stress
    (rheology) and unyielded plugs (rigid bodies), all in one tank; its diluent, water, joins
    the tank's rows though no water particle was placed."""
    sim, ora, problems = run_pair(tanks.yield_stress(mat=6), 16)
    assert not problems, "\n".join(problems[:10])
    st = sim.stats()
    assert st.caps & (1 | 4 | 8 | 64) == (1 | 4 | 8 | 64)
    a, b = sim.field("rl", np.int32).reshape(-1, 2), ora.field("rl", np.int32).reshape(-1, 2)
    assert np.array_equal(a[:, 0], b[:, 0])
