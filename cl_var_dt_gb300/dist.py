"""Multi-rank helpers: chains are independent, so ranks split the chain list
with no data-path collective; the only collective is the max over ranks of the
timed region (and optionally gathering per-rank results on rank 0)."""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple


def rank_world() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def shard_range(n: int, rank: int, world: int) -> range:
    """Contiguous, balanced share of n chains for one rank (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def shard(items: Sequence, rank: int, world: int) -> List:
    return [items[i] for i in shard_range(len(items), rank, world)]


def max_over_ranks(value: float, device=None) -> float:
    """Max of a scalar over the ranks of the default process group (identity
    without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
