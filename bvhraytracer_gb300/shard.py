"""Sharding of the traversal across GPUs (one process per GPU).

Rays are independent and the BVH is read-only, so the work splits into
contiguous ray ranges (or whole scenes) with the scene replicated on every
GPU; no collective is needed on the data path. The only exchange is the
optional sum of counter totals for reports.
"""
from __future__ import annotations


def shard_range(n: int, rank: int, world: int) -> tuple:
    """[begin, end) of the rays of `rank` when `n` rays split over `world`
    ranks as evenly as possible (the first n % world ranks get one more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def reduce_totals(totals, group=None):
    """Sum of per-rank counter totals (a 1-D int64 tensor) over the process
    group, in place; a no-op outside torch.distributed."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(totals, op=dist.ReduceOp.SUM, group=group)
    return totals
