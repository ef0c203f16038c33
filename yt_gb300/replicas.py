"""Replicated volumes across GPUs: split views, gather images.

Rays are independent and a volume fits one GPU's HBM many times over, so
several GPUs each hold a replica of the volume and render a share of the
views; the only communication is gathering finished images to one rank.
(yt's MPI scheme splits the *volume* instead and composites partial images in
kd order, ``amr_kdtree.py:297-323`` -- needed only for volumes larger than one
device.)
"""
from __future__ import annotations

import numpy as np
import torch


def view_cost(resolution) -> int:
    nx, ny = resolution
    return int(nx) * int(ny)


def shard(costs, world: int):
    """Assign items to ranks, greedily balancing total cost (largest first).
    Returns a list of item-index lists, one per rank, each in input order."""
    costs = np.asarray(costs, dtype=np.float64)
    load = np.zeros(world)
    owner = np.empty(costs.size, dtype=np.int64)
    for i in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [sorted(np.nonzero(owner == r)[0].tolist()) for r in range(world)]


def gather_images(images: dict, owner_lists, shapes: dict, rank: int, world: int, dst: int = 0, group=None):
    """Collect ``{view index: (nx, ny, 4) float64 tensor}`` from every rank on
    rank ``dst`` (returns the full dict there, None elsewhere).  ``shapes``
    maps every view index to its image shape (all ranks know the job's
    cameras).  Works with any torch.distributed backend; tensors go through
    the CPU."""
    import torch.distributed as dist

    mine = owner_lists[rank]
    flat = torch.cat([images[i].detach().reshape(-1).cpu() for i in mine]) if mine else torch.zeros(0,
                                                                                                    dtype=torch.float64)
    sizes = torch.tensor([flat.numel()], dtype=torch.int64)
    all_sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(all_sizes, sizes, group=group)
    n_max = int(max(s.item() for s in all_sizes))
    buf = torch.zeros(n_max, dtype=torch.float64)
    buf[: flat.numel()] = flat
    if rank == dst:
        bufs = [torch.zeros(n_max, dtype=torch.float64) for _ in range(world)]
        dist.gather(buf, bufs, dst=dst, group=group)
        out = {}
        for r in range(world):
            off = 0
            for i in owner_lists[r]:
                shape = tuple(shapes[i])
                n = int(np.prod(shape))
                out[i] = bufs[r][off: off + n].reshape(shape)
                off += n
        return out
    dist.gather(buf, None, dst=dst, group=group)
    return None

