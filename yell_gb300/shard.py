"""Splitting a polymul batch across ranks (one process per GPU).

RNS limbs and polymul pairs are independent (no exchange step on the data
path), so a batch is cut into contiguous ranges of pairs, one per rank, each
rank computes its range on its own GPU, and the ranges are reassembled in
order.  The only collective is the optional final gather of results.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_units: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [start, stop) of n_units for `rank`; sizes differ by <= 1."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    q, r = divmod(n_units, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def sharded_polymul(a: np.ndarray, b: np.ndarray, compute, rank: int, world: int, gather=None):
    """Computes this rank's pairs of a (pairs, L, N) batch with `compute(a, b)`
    and, when `gather` is given (a callable that all-gathers one array per
    rank and returns the list in rank order), reassembles the full result."""
    start, stop = shard_range(a.shape[0], rank, world)
    part = compute(np.ascontiguousarray(a[start:stop]), np.ascontiguousarray(b[start:stop]))
    if gather is None:
        return part, (start, stop)
    parts = gather(part)
    return np.concatenate(parts, axis=0), (0, a.shape[0])
