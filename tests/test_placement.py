"""Placement of the batched configuration's tanks over ranks (sprout_gb300.placement): every
tank is placed exactly once, the split is balanced, and two ranks (gloo, world size 2, one
process each on CPU) compute the same partition independently and together cover every tank:
the host-side logic of the multi-GPU path, which exchanges nothing on the data path."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from sprout_gb300 import placement, workloads


def test_partition_places_every_tank_once_and_balances():
    tanks = workloads.uneven_dam_breaks(64, 0)
    for world in (1, 2, 4, 8):
        parts = [placement.my_tanks(tanks, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        costs = [placement.tank_cost(t.w * t.h, 0) for t in tanks]
        assert placement.imbalance(costs, placement.partition(costs, world)) < 1.25


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tanks = workloads.uneven_dam_breaks(64, 0)
        mine = placement.my_tanks(tanks, rank, world)
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)   # host-side check only: nothing on the data path
        out[rank] = everyone
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_partition():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        views = [out[r] for r in range(world)]
    assert views[0] == views[1]
    flat = sorted(i for p in views[0] for i in p)
    assert flat == list(range(64)) and all(len(p) > 0 for p in views[0])
