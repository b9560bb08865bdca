"""The serving loop: scene-step requests over resident tanks, continuous batching.

Tanks are admitted while the device has room (free HBM after a reserve), stay resident
between requests, and every launch advances each tank that has work by one substep: a
request for k substeps of a tank finishes with the k-th launch that includes it. Requests
that arrive while others are on the GPU join the next launch; launches are queued on the
device without waiting (sprout_batch_step_subset) and their completion is polled through
the batch's tickets, so the host keeps forming batches while the device works. Latency is
measured from a request's arrival to the host seeing its last substep done.

    python -m sprout_gb300.serving --scenes 512 --rate 2000 --seconds 60 --precision mixed
"""
from __future__ import annotations

import argparse
import collections
import json
import time

import numpy as np

from . import Batch, device_memory
from .workloads import SERVING_WEIGHTS, uneven_dam_breaks


class Request:
    __slots__ = ("rid", "scene", "substeps", "left", "arrival", "ticket", "done_at")

    def __init__(self, rid, scene, substeps, arrival):
        self.rid, self.scene, self.substeps, self.left, self.arrival = rid, scene, substeps, substeps, arrival
        self.ticket = None
        self.done_at = None


class Server:
    def __init__(self, precision: str = "plain", max_batch: int = 64, reserve_bytes: float = 4e9,
                 max_inflight: int = 2):
        self.batch = Batch([], precision)
        self.max_batch = max_batch
        self.max_inflight = max_inflight       # launches queued on the device at most
        self.completed = 0
        self.reserve = reserve_bytes
        self.sims = []                          # in batch order
        self.live = []                          # live particles per tank
        self.queues = collections.defaultdict(collections.deque)   # tank -> its open requests
        self.order = collections.deque()        # tanks with work, oldest first
        self.inflight = collections.deque()     # requests whose last substep is launched
        self.done = []
        self.next_id = 0
        self.launches = 0
        self.particle_steps = 0

    # ---- admission ---------------------------------------------------------------------
    def admit(self, tank) -> int | None:
        """Makes the tank resident if the device has room for it after the reserve; returns
        its index, or None (refused)."""
        free, _ = device_memory()
        need = tank.w * tank.h * 900 + 4 * tank.w * tank.h * 110   # grid + hierarchy, particles
        if free - need < self.reserve:
            return None
        sim, parts, _ = tank.engine()
        self.batch.add(sim)
        self.sims.append(sim)
        self.live.append(int(np.count_nonzero(parts["kind"])))
        return len(self.sims) - 1

    # ---- requests ----------------------------------------------------------------------
    def submit(self, scene: int, substeps: int, arrival: float) -> Request:
        r = Request(self.next_id, scene, substeps, arrival)
        self.next_id += 1
        q = self.queues[scene]
        if not q:
            self.order.append(scene)
        q.append(r)
        return r

    def pump(self) -> int:
        """One launch: the oldest tanks with work (at most max_batch) advance one substep,
        unless max_inflight launches are still on the device (requests that arrive meanwhile
        then join a larger launch). Returns how many tanks were stepped."""
        n = min(len(self.order), self.max_batch)
        if n == 0:
            return 0
        if self.launches - self.completed >= self.max_inflight:
            self.completed = self.batch.tickets()[1]
            if self.launches - self.completed >= self.max_inflight:
                return 0
        chosen = [self.order.popleft() for _ in range(n)]
        self.batch.step_subset(chosen)
        self.launches += 1
        ticket = self.launches
        for s in chosen:
            self.particle_steps += self.live[s]
            q = self.queues[s]
            r = q[0]
            r.left -= 1
            if r.left == 0:
                q.popleft()
                r.ticket = ticket
                self.inflight.append(r)
            if q:
                self.order.append(s)
        return n

    def poll(self, now: float):
        """Requests whose last launch has finished on the device."""
        _, completed = self.batch.tickets()
        self.completed = completed
        while self.inflight and self.inflight[0].ticket <= completed:
            r = self.inflight.popleft()
            r.done_at = now
            self.done.append(r)

    def drain(self):
        self.batch.sync()
        self.poll(time.perf_counter())


def serving_tanks(n: int, seed: int = 0):
    """The serving mix's resident tanks: grid sizes by the mix's weights (30/25/20/12/8/5 % of
    128 x 72 .. 1024 x 576), seeded dam breaks of one or two liquids from the full-physics
    ranges, as the batched configuration draws them."""
    return uneven_dam_breaks(n, seed, weights=SERVING_WEIGHTS)


def run(scenes: int = 512, rate: float = 2000.0, seconds: float = 60.0, precision: str = "plain",
        max_batch: int = 64, seed: int = 0, max_inflight: int = 2) -> dict:
    """A seeded Poisson stream of scene-step requests (1-8 substeps) over resident tanks."""
    srv = Server(precision, max_batch, max_inflight=max_inflight)
    t0 = time.perf_counter()
    admitted = 0
    for t in serving_tanks(scenes, seed):
        if srv.admit(t) is None:
            break
        admitted += 1
    setup = time.perf_counter() - t0
    rng = np.random.default_rng(seed + 1)
    n_req = int(rate * seconds * 1.2) + 16
    gaps = rng.exponential(1.0 / rate, n_req)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < seconds]
    targets = rng.integers(0, admitted, len(arrivals))
    steps = rng.integers(1, 9, len(arrivals))
    start = time.perf_counter()
    k = 0
    while True:
        now = time.perf_counter() - start
        while k < len(arrivals) and arrivals[k] <= now:
            srv.submit(int(targets[k]), int(steps[k]), float(arrivals[k]))
            k += 1
        srv.poll(time.perf_counter() - start)
        stepped = srv.pump()
        if k >= len(arrivals) and not srv.order:
            break
        if not stepped:
            if srv.order:   # the device is busy: check again shortly
                time.sleep(2e-5)
            elif k < len(arrivals):
                time.sleep(max(0.0, min(arrivals[k] - (time.perf_counter() - start), 0.001)))
    srv.batch.sync()
    end = time.perf_counter() - start
    srv.poll(end)
    lat = np.array([(r.done_at - r.arrival) * 1e3 for r in srv.done])
    return {"scenes": admitted, "requests": len(srv.done), "offered_rate": rate, "seconds": seconds,
            "wall_s": end, "setup_s": setup, "launches": srv.launches,
            "mean_batch": float(sum(steps[: len(srv.done)]) / max(srv.launches, 1)),
            "particle_steps_per_s": srv.particle_steps / end,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "precision": precision, "max_batch": max_batch, "max_inflight": max_inflight}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--seconds", type=float, default=60.0)
    ap.add_argument("--precision", default="plain", choices=["plain", "mixed"])
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--max-inflight", type=int, default=2)
    a = ap.parse_args()
    print(json.dumps(run(a.scenes, a.rate, a.seconds, a.precision, a.max_batch, a.seed, a.max_inflight)), flush=True)


if __name__ == "__main__":
    main()
