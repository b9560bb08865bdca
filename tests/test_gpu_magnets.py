"""Magnets on the GPU, bit for bit against the oracle: the field of the dipoles, the energy
density with and without the demagnetising factor, the face forces (magnet.comp), the
susceptibility and the magnetic resting rule of grid prep; a magnet tank in a batch as alone."""
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mat,demag", [(37, 0.0), (13, 0.5)])
def test_magnets_bit_exact(mat, demag):
    sim, ora, problems = run_pair(tanks.magnetic(mat=mat, demag=demag), 16)
    assert not problems, "\n".join(problems[:10])
    n, k = first_diff(sim.field("magc"), ora.field("magc"))
    assert n == 0, f"magc differs in {n} values (first {k})"


def test_magnet_tank_in_a_batch_equals_alone():
    def variants():
        return [tanks.magnetic(mat=37), tanks.magnetic(128, 72, mat=13, demag=0.5), tanks.dam_break(96, 64)]
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
