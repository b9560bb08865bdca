"""Batched stepping (sprout_batch_*): tanks of different sizes and physics advanced together by
one graph per substep, their pressure solves in one persistent kernel over all their tiles.
The batch changes scheduling only: every tank must come out bit for bit as it does stepping
alone (the same tile arithmetic, the same reduction order per tank)."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from test_gpu_parity import GRID_FIELDS, by_id, first_diff

pytestmark = pytest.mark.gpu


def mix():
    return [tanks.dam_break(96, 64), tanks.dam_break(128, 72, width=0.6, height=0.5),
            tanks.stratified(128, 72), tanks.full_physics(160, 96, cell=0.0064)]


def compare(a, b, tag):
    msgs = []
    pa, pb = by_id(a.download_particles()), by_id(b.download_particles())
    if not np.array_equal(pa.view(np.uint8), pb.view(np.uint8)):
        msgs.append(f"{tag}: particles differ")
    for name in GRID_FIELDS:
        n, k = first_diff(a.field(name), b.field(name))
        if n:
            msgs.append(f"{tag}: {name} differs in {n} values")
    sa, sb = a.stats(), b.stats()
    for f in ["pressure_iters_max", "pressure_unconverged", "pressure2_iters_max", "viscosity_iters_max",
              "solves", "pressure_residual_max"]:
        if getattr(sa, f) != getattr(sb, f):
            msgs.append(f"{tag}: {f} {getattr(sa, f)} vs {getattr(sb, f)}")
    return msgs


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_batch_equals_alone(precision):
    alone = [t.engine()[0] for t in mix()]
    for s in alone:
        s.set_precision(precision)
    batched = [t.engine()[0] for t in mix()]
    batch = S.Batch(batched, precision)
    n = 10
    for s in alone:
        s.step(n, n / 240.0)
    batch.step(n)
    batch.sync()
    problems = []
    for k, (a, b) in enumerate(zip(alone, batched)):
        problems += compare(a, b, f"tank {k}")
    assert not problems, "\n".join(problems)
    st = batched[2].stats()
    assert st.viscosity_mode == 2 and st.pressure2_iters_max > 0


def test_batch_viscosity_variants_equal_alone():
    """The implicit viscosity before a single pressure solve (viscous_projection 0: its solve
    runs inside the grid stage, on the batch's main stream), the Jacobi-preconditioned solve
    (one solve per tank), and multigrid-preconditioned tanks solved together in one batched
    viscosity kernel: each tank as it steps alone."""
    def variants():
        return [tanks.stratified(128, 72, extra={"viscous_projection": 0}),
                tanks.stratified(96, 64, extra={"viscosity_precond": 0}),
                tanks.stratified(128, 72), tanks.full_physics(160, 96, cell=0.0064),
                tanks.dam_break(96, 64)]
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
    st = [s.stats() for s in batched]
    assert st[0].viscosity_mode == 2 and st[0].pressure2_iters_max == 0
    assert st[1].viscosity_iters_max > st[2].viscosity_iters_max > 0


def test_batch_membership_changes():
    """Adding and removing tanks between steps re-records the batch; a removed tank steps
    alone again."""
    ts = mix()
    sims = [t.engine()[0] for t in ts]
    batch = S.Batch(sims[:2])
    batch.step(3)
    batch.add(sims[2])
    batch.step(2)
    batch.remove(sims[0])
    batch.step(2)
    batch.sync()
    sims[0].step(1, 1 / 240.0)
    assert sims[0].stats().substeps == 6
    assert sims[1].stats().substeps == 7 and sims[2].stats().substeps == 4
