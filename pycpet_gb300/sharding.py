"""Multi-GPU host logic: frames shard across ranks with no exchange.

Frames, grid points and streamlines are independent, so a job of many frames
is split by frame over the ranks (one process per GPU) and nothing crosses
ranks on the data path.  The only collective is the timing reduction: the
job's time is the slowest rank's.
"""
from __future__ import annotations

import numpy as np


def shard_frames(costs, rank: int, world: int):
    """Frame indices of `rank`: longest-processing-time-first assignment of
    per-frame costs (e.g. pair evaluations) to `world` ranks, deterministic
    on every rank."""
    costs = np.asarray(costs, dtype=np.float64)
    if world <= 1:
        return list(range(len(costs)))
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [int(i) for i in np.flatnonzero(owner == rank)]


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over all ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
