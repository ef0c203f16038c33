"""Replicas across ranks (CPU, gloo, world size 2): views are split by cost
and the gathered images equal a single-rank run."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from yt_gb300.replicas import gather_images, shard, view_cost


def test_shard_balances_and_covers():
    rng = np.random.default_rng(0)
    res = [(int(a), int(a)) for a in rng.choice([128, 256, 512, 1024], 64)]
    costs = [view_cost(r) for r in res]
    parts = shard(costs, 4)
    assert sorted(sum(parts, [])) == list(range(64))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def fake_render(i, shape):
    # a deterministic "image" per view, standing in for a GPU render
    g = torch.Generator().manual_seed(1000 + i)
    return torch.rand(shape, generator=g, dtype=torch.float64)


def _worker(rank, world, port, shapes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        parts = shard([view_cost(s[:2]) for s in shapes.values()], world)
        mine = {i: fake_render(i, shapes[i]) for i in parts[rank]}
        out = gather_images(mine, parts, shapes, rank, world)
        if rank == 0:
            q.put({k: v.numpy() for k, v in out.items()})
    finally:
        dist.destroy_process_group()


def test_two_rank_gather_matches_single_rank():
    shapes = {i: (8 + 4 * (i % 3), 6 + 2 * (i % 2), 4) for i in range(7)}
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, shapes, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(got) == list(range(7))
    for i, s in shapes.items():
        assert np.array_equal(got[i], fake_render(i, s).numpy())
