"""Ket-block sharding across ranks (one process per GPU).

The path shards over kets with no exchange while stepping: rank r evolves kets
[lo_r, hi_r) of the block.  Readouts that sum over kets (local densities, bond currents,
particle number) are the only cross-rank step: an all-reduce (sum) of an N- or
bond-length FP64 vector through torch.distributed.
"""
from __future__ import annotations

import numpy as np


def shard_range(M: int, rank: int, world: int):
    """Contiguous, balanced ket range [lo, hi) of `rank` (the first M % world ranks get one more)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(M, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def allreduce_sum(values: np.ndarray, group=None) -> np.ndarray:
    """Sums an FP64 vector over ranks (in place semantics on a copy); identity without a group."""
    import torch
    import torch.distributed as dist
    v = np.ascontiguousarray(values, dtype=np.float64)
    if not dist.is_available() or not dist.is_initialized():
        return v.copy()
    backend = dist.get_backend(group)
    t = torch.from_numpy(v.copy())
    if backend == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
