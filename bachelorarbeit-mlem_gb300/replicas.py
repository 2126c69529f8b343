"""Independent replicas across GPUs (one process per GPU).

The MLEM path does not need a collective on one GPU; across GPUs the
reconstructions are independent, so the work is sharded by instance: every
rank reconstructs a contiguous, balanced block of the sinograms on its own
GPU and the images are gathered on rank 0 in submission order.  No data-path
collective is involved; torch.distributed only carries the finished images.
"""
from __future__ import annotations

from typing import Callable, Sequence


def shard(count: int, rank: int, world: int) -> range:
    """Contiguous block of [0, count) owned by rank (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def run_sharded(fn: Callable[[int], object], count: int, group=None) -> list | None:
    """Runs fn(i) for this rank's block; rank 0 receives all results in order."""
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = [(i, fn(i)) for i in shard(count, rank, world)]
    if world == 1:
        return [r for _, r in mine]
    gathered: Sequence = [None] * world if rank == 0 else None
    dist.gather_object(mine, gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * count
    for part in gathered:
        for i, r in part:
            out[i] = r
    return out
