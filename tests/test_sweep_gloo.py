"""Aero-map case list and its split over ranks, checked with two gloo processes
on CPU: every case runs exactly once, the serpentine order is the reference's
(src/ui/aeromap.ts:79-84), and the max-over-ranks timing reduction works."""
import os
import socket

import pytest

from windtunnel.sweep import aero_map_points, serpentine, shard


def test_serpentine_order():
    assert serpentine(2, 3) == [(0, 0), (0, 1), (0, 2), (1, 2), (1, 1), (1, 0)]
    pts = aero_map_points()
    assert len(pts) == 25
    assert [p.front for p in pts[:5]] == [0.010] * 5
    assert [p.rear for p in pts[5:10]] == [0.060, 0.0475, 0.035, 0.0225, 0.010]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard(aero_map_points(), rank, world)
    got = [None] * world
    dist.all_gather_object(got, [p.index for p in mine])
    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((got, float(t.item())))
    dist.destroy_process_group()


def test_two_rank_split():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    flat = sorted(i for part in got for i in part)
    assert flat == list(range(25))
    assert abs(len(got[0]) - len(got[1])) <= 1
    assert tmax == 2.0
