"""Non-Newtonian liquids on the GPU, bit for bit against the oracle: grid prep's record of each
cell's non-Newtonian liquid and the rigid-viscosity cap (grid_prep.comp:162, 210, 232-237),
rheo.comp's viscosity from the shear rate with the engine's own ln / exp (common.glsl:527-571),
and the implicit viscosity that follows; a shear-thinning tank in a batch as alone."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_batch import compare
from test_gpu_parity import first_diff, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mat", [7, 19])
def test_shear_thinning_bit_exact(mat):
    sim, ora, problems = run_pair(tanks.shear_thinning(mat=mat), 12)
    assert not problems, "\n".join(problems[:10])
    for name in ["rh", "cell"]:
        n, k = first_diff(sim.field(name), ora.field(name))
        assert n == 0, f"{name} differs in {n} values (first {k})"
    rh = sim.field("rh").reshape(-1, 4)
    assert np.count_nonzero(rh[:, 0] > 0) > 500


def test_shear_thinning_in_a_batch_equals_alone():
    def variants():
        return [tanks.shear_thinning(mat=7), tanks.shear_thinning(128, 72, mat=19), tanks.dam_break(96, 64)]
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
