"""Several phase groups on the GPU, bit for bit against the oracle: the particle pass's drift
between groups and within one (particles.comp:374-502), the group fields of grid prep (aux,
grho, gbase: grid_prep.comp:53, 172, 247-252), the per-group curvature and pair jumps of the
surface passes; and such tanks stepping in a batch as they step alone."""
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


def fields_agree(sim, ora, names):
    bad = []
    for name in names:
        a, b = sim.field(name), ora.field(name)
        n, k = first_diff(a, b)
        if n:
            bad.append(f"{name} differs in {n} values (first {k})")
    return bad


def test_water_and_oil_bit_exact():
    sim, ora, problems = run_pair(tanks.water_oil(), 16)
    assert not problems, "\n".join(problems[:10])
    assert not fields_agree(sim, ora, ["aux", "grho", "surf2", "pjump"])


def test_three_groups_with_sorting_bit_exact():
    sim, ora, problems = run_pair(tanks.three_groups(), 16)
    assert not problems, "\n".join(problems[:10])
    assert not fields_agree(sim, ora, ["aux", "grho", "gbase", "surf2", "pjump"])


def test_group_tanks_in_a_batch_equal_alone():
    def variants():
        return [tanks.water_oil(), tanks.three_groups(128, 72), tanks.honey_dam()]
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


def test_builtin_liquids_bit_exact():
    """Water, ink and milk (two families), olive oil and mercury (three groups): the built-in
    rows as the reference's table has them."""
    sim, ora, problems = run_pair(tanks.builtin_mix(), 12)
    assert not problems, "\n".join(problems[:10])
    assert not fields_agree(sim, ora, ["aux", "grho", "mixb"])
