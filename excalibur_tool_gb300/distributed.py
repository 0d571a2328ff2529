"""Photon sharding across ranks (one process per GPU, full replica of every grid).

Photons are independent ODEs, so a multi-GPU run needs no collective on the data
path: each rank traces a contiguous slice of the photon index range (the reference's
process pool splits its photon list the same way, integration/integrator.py:443-473)
and the slices are gathered once at the end. Works with any torch.distributed
backend (NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations


def shard_range(n: int, rank: int, world: int):
    """[start, stop) of rank's slice: sizes differ by at most one, in rank order."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("need world >= 1, 0 <= rank < world, n >= 0")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_rows(local, n: int, group=None):
    """All ranks' row slices (shard_range order) concatenated into the full [n, ...] tensor on every rank.

    `local` is this rank's slice (a tensor on the device the backend uses)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    sizes = [shard_range(n, r, world) for r in range(world)]
    width = max(b - a for a, b in sizes)
    pad = torch.zeros((width, *local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[: b - a] for p, (a, b) in zip(parts, sizes)])
