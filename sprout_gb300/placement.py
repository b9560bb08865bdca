"""Placement of many tanks over several GPUs: the batched and serving configurations' tanks are
independent units (one tank does not shard: every CG iteration has two global reductions
and every smoother sweep a halo exchange), so they are partitioned across ranks, one process
per GPU, with no collective on the data path; only statistics and latencies are gathered on
the host.

The partition is greedy bin packing on each tank's cost, cells + particles / 4 (the pressure
and viscosity solves scale with cells, the particle passes with particles at about a quarter
of a cell's bytes): tanks in decreasing cost, each to the rank with the least cost so far
(ties to the lower rank). Every rank computes the same partition from the same list, so no
exchange is needed to agree on it.
"""
from __future__ import annotations


def tank_cost(cells: int, particles: int) -> float:
    return float(cells) + 0.25 * float(particles)


def partition(costs: list[float], ranks: int) -> list[list[int]]:
    """Indices of the tanks each rank takes (each list in ascending order)."""
    if ranks < 1:
        raise ValueError("ranks >= 1")
    load = [0.0] * ranks
    out = [[] for _ in range(ranks)]
    for k in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(ranks), key=lambda j: (load[j], j))
        out[r].append(k)
        load[r] += costs[k]
    return [sorted(o) for o in out]


def imbalance(costs: list[float], parts: list[list[int]]) -> float:
    """Largest rank's cost over the mean: 1 is a perfect split."""
    loads = [sum(costs[i] for i in p) for p in parts]
    mean = sum(loads) / max(len(loads), 1)
    return max(loads) / mean if mean > 0 else 1.0


def my_tanks(tanks: list, rank: int, world: int) -> list[int]:
    """The indices of `tanks` (workload descriptions) this rank steps."""
    costs = [tank_cost(t.w * t.h, sum(int((r[2] - r[0]) * (r[3] - r[1]) * 4) for r, _, _ in t.fills)) for t in tanks]
    return partition(costs, world)[rank]
