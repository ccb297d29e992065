"""Data-parallel replicas: one process per GPU, structures split between ranks.

Structures are independent in this path, so a batch spreads over ranks with no
exchange on the data path: each rank evaluates its own share (contiguous ranges,
balanced by atom count) and the results come back together in the caller's
order.  The only collectives are the result gather and the timing reduction
(the slowest rank's time), both on the host side of the step.
"""
from __future__ import annotations

import numpy as np


def shard(natoms_per_structure, rank, world):
    """Indices of the structures rank `rank` of `world` evaluates: contiguous ranges
    whose atom counts are as equal as the structure boundaries allow."""
    n = np.asarray(natoms_per_structure, dtype=np.int64)
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    if len(n) == 0:
        return np.zeros(0, dtype=np.int64)
    cum = np.concatenate([[0], np.cumsum(n)])
    total = cum[-1]
    # structure s goes to the rank whose share of the atom count holds its midpoint
    mid = (cum[:-1] + cum[1:]) / 2.0
    owner = np.minimum((mid * world / max(total, 1)).astype(np.int64), world - 1)
    return np.nonzero(owner == rank)[0]


def gather(local, indices, group=None):
    """Collect per-structure results from all ranks into the caller's order.

    local: list of per-structure results of this rank (any picklable objects), in the
    order of `indices` (this rank's structure indices).  Returns the full list on
    every rank."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (list(map(int, indices)), list(local)), group=group)
    n = sum(len(ix) for ix, _ in parts)
    out = [None] * n
    for ix, res in parts:
        for i, r in zip(ix, res):
            out[i] = r
    return out


def max_over_ranks(value, device=None, group=None):
    """The largest value over the ranks (the slowest rank's time); value itself with
    one process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
