"""The frame pacer (sprout_pacer_*, src/pacing.rs) against the reference's own tests of it
(pacing.rs:114-203), restated with their frame model and assertions: a light scene keeps real
time, a heavy one slows time with an even frame time, short frames bank time for full-length
substeps, a hitch is not paid back, slow motion scales the substep count."""
import numpy as np
import pytest

import sprout_gb300 as S

F = np.float32
DT = F(1.0) / F(240.0)
BUDGET = F(0.8) / F(60.0)


@pytest.fixture(autouse=True)
def _lib(engine_lib):
    return engine_lib


def run(pacer, overhead, cost, dt, vsync, frames):
    """Frames of a fixed overhead plus a cost per substep (pacing.rs:121-138), in f32."""
    simulated, wall = F(0.0), F(0.0)
    times = []
    frame_dt = max(F(vsync), F(overhead))
    for frame in range(frames):
        plan = pacer.plan(float(frame_dt), float(dt), False, 1.0, float(cost), float(BUDGET))
        work = F(overhead) + F(plan.substeps) * F(cost)
        frame_dt = F(max(np.ceil(work / F(vsync)), F(1.0)) * F(vsync)) if vsync > 0.0 else work
        simulated = F(simulated + F(plan.expected))
        wall = F(wall + frame_dt)
        if frame > frames // 2:
            times.append(float(frame_dt))
    return float(simulated), float(wall), times


def test_a_light_scene_runs_in_real_time():
    for vsync in [0.0, 1.0 / 60.0, 1.0 / 165.0]:
        pacer = S.Pacer()
        simulated, wall, _ = run(pacer, 0.0005, 0.001, DT, vsync, 4000)
        assert abs(simulated / wall - 1.0) < 0.02, (vsync, simulated, wall)
        assert abs(pacer.speed() - 1.0) < 0.1, (vsync, pacer.speed())


def test_a_heavy_scene_slows_time_and_keeps_an_even_frame_time():
    # 6 ms per substep of 1/240 s: real time would need 1.44 s of work per second
    for vsync in [0.0, 1.0 / 60.0]:
        pacer = S.Pacer()
        simulated, wall, times = run(pacer, 0.001, 0.006, DT, vsync, 2000)
        lo, hi = min(times), max(times)
        assert hi < 1.0 / 55.0, (vsync, hi)
        assert hi - lo < 1e-4, (vsync, lo, hi)
        speed = simulated / wall
        assert 0.4 < speed < 0.75, (vsync, speed)
        assert abs(pacer.speed() - speed) < 0.15


def test_short_frames_bank_time_for_full_length_substeps():
    # uncapped: 0.4 ms frames, 5 ms substeps that cost 3 ms each
    pacer = S.Pacer()
    dt = 0.005
    steps, simulated, frame_dt = 0, F(0.0), F(0.0004)
    for _ in range(5000):
        plan = pacer.plan(float(frame_dt), dt, False, 1.0, 0.003, float(BUDGET))
        assert plan.substeps <= 1
        steps += plan.substeps
        simulated = F(simulated + F(plan.expected))
        frame_dt = F(0.0004) + F(plan.substeps) * F(0.003)
    mean = float(simulated) / steps
    assert mean > 0.85 * dt, mean


def test_a_hitch_is_not_paid_back():
    pacer = S.Pacer()
    run(pacer, 0.0005, 0.001, DT, 1.0 / 60.0, 200)
    # half a second without a frame must not turn into a burst of catch-up substeps
    n = pacer.plan(0.5, float(DT), False, 1.0, 0.001, float(BUDGET)).substeps
    assert n <= 24
    nxt = pacer.plan(1.0 / 60.0, float(DT), False, 1.0, 0.001, float(BUDGET)).substeps
    assert nxt <= 5, nxt


def test_slow_motion_scales_the_substep_count():
    pacer = S.Pacer()
    total = sum(pacer.plan(1.0 / 60.0, float(DT), False, 0.25, 0.001, float(BUDGET)).substeps for _ in range(600))
    assert abs(total - 600) <= 12, total
    assert abs(pacer.speed() - 1.0) < 0.1


def test_fixed_rate_and_reset():
    pacer = S.Pacer()
    p = pacer.plan(1.0 / 60.0, float(DT), True, 1.0, 0.0, float(BUDGET))
    assert p.substeps == 2 and p.target == p.expected   # unmeasured: at most two substeps
    pacer.reset()
    p = pacer.plan(1e-4, float(DT), True, 1.0, 0.0, float(BUDGET))
    assert p.substeps == 0 and p.target == 0.0
