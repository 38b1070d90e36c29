"""Sharding of independent trees across ranks (one process per GPU).

The PMM path has no exchange step: candidate trees, serving requests and EM
restarts are independent, so each rank takes a contiguous shard, runs its
own batch, and rank 0 gathers the per-tree results in the original order.
The timing rule of a weak-scaling run is the maximum over ranks.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import torch
import torch.distributed as dist


def shard_bounds(n_items: int, rank: int, world: int) -> Tuple[int, int]:
    """[lo, hi) of rank's contiguous shard; shards differ in size by <= 1."""
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(items: Sequence, rank: int, world: int) -> List:
    lo, hi = shard_bounds(len(items), rank, world)
    return list(items[lo:hi])


def gather_scores(local: Sequence[float], n_items: int, group=None) -> List[float]:
    """All-gather every rank's per-tree scores into one list in item order
    (host tensors; works with gloo on CPU and NCCL on GPU tensors)."""
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_bounds(n_items, rank, world)
    buf = torch.zeros(n_items, dtype=torch.float64)
    buf[lo:hi] = torch.as_tensor(list(local), dtype=torch.float64)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    return buf.tolist()


def max_over_ranks(seconds: float, group=None) -> float:
    t = torch.tensor([seconds], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
