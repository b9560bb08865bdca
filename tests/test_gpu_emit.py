"""The brush's emitters on the device (sprout_sim_emit_stream / _paint / _rain) against the
CPU restatement of World::emit and brush.rs (oracle/brush.py), bit for bit: two copies of a
tank, one fed by the device emitters, the other by the restatement's particles through the
engine's host spawn path (which is itself pinned to the oracle); after every emission the
live particles (position, velocity, concentration, kind, id, temperature) agree by id, and
they keep agreeing through the substeps that follow (the CFL limit of a step call included,
which the fastest emitted particle raises)."""
import numpy as np
import pytest

import sprout_gb300 as S
import tanks
from oracle import brush as B

pytestmark = pytest.mark.gpu


def live_by_id(sim):
    p = sim.download_particles()
    p = p[(p["kind"] & 255) != 0]
    return np.sort(p, order="id")


def same(a, b):
    if len(a) != len(b):
        return f"{len(a)} live particles against {len(b)}"
    bad = np.flatnonzero(np.any(a.view(np.uint32).reshape(len(a), -1) != b.view(np.uint32).reshape(len(b), -1), axis=1))
    return None if len(bad) == 0 else f"{len(bad)} particles differ, first id {a['id'][bad[0]]}: {a[bad[0]]} vs {b[bad[0]]}"


def pair(tank):
    a, parts, (sdf, _, _, _) = tank.engine()
    b, _, _ = tank.engine()
    world = B.World(tank.w, tank.h, sdf, lambda lo, hi: b.cell_counts(lo, hi).ravel())
    return a, b, world


def spawn_host(sim, out, material):
    if not out:
        return 0
    p = np.zeros(len(out), S.PARTICLE_DTYPE)
    for k, (pos, vel) in enumerate(out):
        p["pos"][k] = pos
        p["vel"][k] = vel
    p["s"] = -1.0            # SPAWN_S
    p["t"] = -1.0e4          # SPAWN_TEMP
    p["kind"] = material + 1
    return sim.spawn(p)


def check(a, b, what):
    a.step_blocking(0)
    b.step_blocking(0)
    msg = same(live_by_id(a), live_by_id(b))
    assert msg is None, f"{what}: {msg}"


def obstacle_tank(fixed=True):
    t = tanks.dam_break(160, 96, width=0.3, height=0.4)
    t.shapes = [{"kind": "box", "c": [95.0, 55.0], "half": [8.0, 3.0], "angle": 0.3}]
    if not fixed:
        t.settings.pop("fixed_hz", None)
    return t


def test_every_source_matches_the_restatement():
    t = obstacle_tank()
    a, b, world = pair(t)
    dt = 1 / 240.0
    total = 0
    # a stamp (World::stamp: a full disk of rest-density liquid where there is none)
    a.emit_paint((120.0, 30.0), (120.0, 30.0), 6.0, 32768, False, 0)
    out = world.paint((120.0, 30.0), (120.0, 30.0), 6.0, 32768, False)
    total += spawn_host(b, out, 0)
    check(a, b, "stamp")
    # a pour moving over the obstacle for a few frames, substeps between
    sp = S.Spout.make("pour", 6000.0, 5.0)
    osp = B.Spout.pour(6000.0, 5.0)
    sa, so = S.StreamState(), B.Stream()
    x = 80.0
    for f in range(4):
        frm, to = (x, 85.0), (x + 3.0, 85.0)
        a.emit_stream(sp, sa, frm, to, 1 / 60.0, 0)
        total += spawn_host(b, world.stream(so, osp, frm, to, 1 / 60.0), 0)
        check(a, b, f"pour frame {f}")
        a.step(2, 2 * dt)
        b.step(2, 2 * dt)
        x += 3.0
    assert sa.time == so.time
    # particles queued by the host spawn before an emission take their ids first
    extra = [((f32x, 88.0), (0.0, -5.0)) for f32x in np.linspace(60.0, 70.0, 12, dtype=np.float32)]
    spawn_host(a, extra, 0)
    total_host = spawn_host(b, extra, 0)
    # spray along a stroke, then rain, a jet, another material (a new row of the tank)
    a.emit_paint((30.0, 70.0), (45.0, 72.0), 6.0, 300, True, 0)
    total += spawn_host(b, world.paint((30.0, 70.0), (45.0, 72.0), 6.0, 300, True), 0)
    check(a, b, "spray")
    a.emit_rain((120.0, 80.0), 5.0, 120, 0)
    total += spawn_host(b, world.rain((120.0, 80.0), 5.0, 120), 0)
    check(a, b, "rain")
    jet = S.Spout.make("jet", 8000.0, 4.0, 70.0)
    ojet = B.Spout.jet(70.0, 8000.0, 4.0)
    ja, jo = S.StreamState(), B.Stream()
    a.emit_stream(jet, ja, (20.0, 50.0), (20.0, 50.0), 1 / 30.0, 2)
    total += spawn_host(b, world.stream(jo, ojet, (20.0, 50.0), (20.0, 50.0), 1 / 30.0), 2)
    check(a, b, "jet of oil")
    assert a.emitted()[0] == total and total > 500 and total_host == 12
    for _ in range(3):
        a.step(2, 2 * dt)
        b.step(2, 2 * dt)
    msg = same(live_by_id(a), live_by_id(b))
    assert msg is None, f"after the substeps: {msg}"


def test_the_fastest_emitted_particle_limits_the_next_step_call():
    """Without a fixed rate the substep comes from the CFL limit, which the spawned particles'
    fastest speed raises for the next step call (mod.rs:2300): the same dt in both copies."""
    t = obstacle_tank(fixed=False)
    a, b, world = pair(t)
    jet = S.Spout.make("jet", 8000.0, 4.0, 100.0)
    ojet = B.Spout.jet(100.0, 8000.0, 4.0)
    ja, jo = S.StreamState(), B.Stream()
    for f in range(3):
        a.emit_stream(jet, ja, (20.0, 60.0), (20.0, 60.0), 1 / 60.0, 0)
        spawn_host(b, world.stream(jo, ojet, (20.0, 60.0), (20.0, 60.0), 1 / 60.0), 0)
        a.step(3, 1 / 60.0)
        b.step(3, 1 / 60.0)
        sa, sb = a.stats(), b.stats()
        assert sa.dt == sb.dt and sa.dt_prev == sb.dt_prev, (f, sa.dt, sb.dt)
    msg = same(live_by_id(a), live_by_id(b))
    assert msg is None, msg


def test_a_blocked_spout_admits_nothing_and_leaves_dead_slots():
    """A spout inside a solid admits nothing; the fresh slots reserved for it stay dead, and
    what is emitted later claims them (the tank's spare capacity is smaller than the stream's
    candidates, so the reserve takes all of it)."""
    t = tanks.dam_break(96, 64, width=0.5, height=0.5)
    t.shapes = [{"kind": "box", "c": [70.0, 30.0], "half": [12.0, 12.0], "angle": 0.0}]
    a, b, world = pair(t)
    n0 = a.stats().n_slots
    sp = S.Spout.make("pour", 3000.0, 3.0)
    a.emit_stream(sp, S.StreamState(), (70.0, 30.0), (70.0, 30.0), 1 / 60.0, 0)
    out = world.stream(B.Stream(), B.Spout.pour(3000.0, 3.0), (70.0, 30.0), (70.0, 30.0), 1 / 60.0)
    assert a.emitted() == (0, 0) and len(out) == 0
    check(a, b, "blocked spout")
    assert a.stats().n_slots > n0   # the reserve, left dead
    a.emit_paint((30.0, 55.0), (30.0, 55.0), 3.0, 32768, False, 0)
    n = spawn_host(b, world.paint((30.0, 55.0), (30.0, 55.0), 3.0, 32768, False), 0)
    assert n > 0 and a.emitted()[0] == n
    check(a, b, "a stamp into the reserve")
