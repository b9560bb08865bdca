"""Viscoelastic liquids on the GPU, bit for bit against the oracle: the particles' stress
update and its move through the sort, its deposit (three fixed-point channels), the grid's
stress and elastic.comp's forces; an elastic tank in a batch as alone."""
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mat", [12, 33])
def test_elastic_bit_exact(mat):
    sim, ora, problems = run_pair(tanks.elastic_drop(mat=mat), 16)
    assert not problems, "\n".join(problems[:10])
    n, k = first_diff(sim.field("estr"), ora.field("estr"))
    assert n == 0, f"estr differs in {n} values (first {k})"


def test_elastic_tank_in_a_batch_equals_alone():
    def variants():
        return [tanks.elastic_drop(mat=12), tanks.elastic_drop(128, 72, mat=33), tanks.dam_break(96, 64)]
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
