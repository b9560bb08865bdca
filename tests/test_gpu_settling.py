"""Settling suspensions on the GPU, bit for bit against the oracle: the family occupancy of
grid prep, settle.comp's gain / loss rates, and the particles taking them (with mud, the
shear-thinning viscosity as well); a settling tank in a batch as alone."""
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mat", [51, 3])
def test_settling_bit_exact(mat):
    sim, ora, problems = run_pair(tanks.settling(mat=mat), 16)
    assert not problems, "\n".join(problems[:10])
    for name in ["famocc", "dsettle"]:
        a, b = sim.field(name), ora.field(name)
        assert a.size == b.size > 0
        n, k = first_diff(a, b)
        assert n == 0, f"{name} differs in {n} values (first {k})"


def test_settling_in_a_batch_equals_alone():
    def variants():
        return [tanks.settling(mat=51), tanks.settling(128, 72, mat=3), tanks.dam_break(96, 64)]
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
