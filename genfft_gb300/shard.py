"""Batch sharding across GPUs.

Batched transforms are independent, so N GPUs split a batch into contiguous
slices with no exchange between them.  Slice sizes differ by at most one.
"""
from __future__ import annotations


def shard_range(batch: int, rank: int, world: int) -> tuple[int, int]:
    """(first index, count) of rank's contiguous slice of `batch` items."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)
