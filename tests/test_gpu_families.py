"""Concentration families on the GPU, bit for bit against the oracle: the particle pass's
family gather, miscible exchange and joining (particles.comp:288-569), the per-family cell
concentrations of grid prep (grid_prep.comp:67-68, 141-147), and a family tank stepping in a
batch as it steps alone."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


def test_honey_family_bit_exact():
    sim, ora, problems = run_pair(tanks.honey_dam(), 16)
    assert not problems, "\n".join(problems[:10])
    p = ora.particles()
    live = p[p["kind"] != 0]
    assert np.any(((live["kind"] & 255) == 2) & (live["s"] < 1.0)), "the exchange ran"


def test_several_families_bit_exact():
    sim, ora, problems = run_pair(tanks.families_tank(), 16)
    assert not problems, "\n".join(problems[:10])
    a, b = sim.field("mixb"), ora.field("mixb")
    assert a.size == b.size > 0
    n, k = first_diff(a, b)
    assert n == 0, f"mixb differs in {n} values (first {k})"


def test_stratified_honey_family_bit_exact():
    sim, ora, problems = run_pair(tanks.stratified(128, 72, builtins=True), 8)
    assert not problems, "\n".join(problems[:10])


def test_family_tanks_in_a_batch_equal_alone():
    def variants():
        return [tanks.families_tank(), tanks.honey_dam(128, 72), tanks.dam_break(96, 64)]
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
