"""The serving loop (sprout_gb300.serving): requests over resident tanks, continuous batching
through sprout_batch_step_subset. Each tank must come out exactly as the same tank stepped
alone by as many substeps as its requests asked for, whatever it was batched with: alone one
substep per step call, since each served launch is a frame of one substep (the recorded
iteration counts adapt per frame)."""
import numpy as np
import pytest

import tanks
from sprout_gb300.serving import Server
from test_gpu_batch import compare

pytestmark = pytest.mark.gpu


def kinds():
    return [tanks.dam_break(96, 64), tanks.dam_break(128, 72, width=0.6, height=0.5),
            tanks.stratified(128, 72), tanks.dam_break(160, 96, width=0.3, height=0.7),
            tanks.full_physics(160, 96, cell=0.0064)]


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_results_same_alone_and_in_the_mix(precision):
    ts = kinds()
    srv = Server(precision, max_batch=3, reserve_bytes=0)
    for t in ts:
        assert srv.admit(t) is not None
    rng = np.random.default_rng(5)
    total = [0] * len(ts)
    for k in range(24):
        s = int(rng.integers(0, len(ts)))
        n = int(rng.integers(1, 5))
        total[s] += n
        srv.submit(s, n, 0.0)
        if k % 3 == 0:
            srv.pump()
    while srv.order:
        srv.pump()
    srv.drain()
    assert len(srv.done) == 24 and not srv.inflight
    problems = []
    for k, t in enumerate(ts):
        alone = t.engine()[0]
        alone.set_precision(precision)
        for _ in range(total[k]):   # one substep per call: each served launch is a frame of one
            alone.step(1, 1 / 240.0)
        assert srv.sims[k].stats().substeps == total[k]
        problems += compare(alone, srv.sims[k], f"tank {k}")
    assert not problems, "\n".join(problems)


def test_tickets_track_completion():
    srv = Server("plain", max_batch=2, reserve_bytes=0)
    for t in kinds()[:3]:
        srv.admit(t)
    for s in range(3):
        srv.submit(s, 2, 0.0)
    while srv.order:
        srv.pump()
    issued, _ = srv.batch.tickets()
    assert issued == srv.launches == 3
    srv.drain()
    assert srv.batch.tickets() == (3, 3)
    assert [r.rid for r in srv.done] == sorted(r.rid for r in srv.done)
