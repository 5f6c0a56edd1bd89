"""Splitting independent replicas between GPUs (one process per GPU).

The step loop of a replica never reads another replica's data, so a batch is
split between ranks with no data exchange: each rank builds a `SystemBatch` of
its share and steps it alone. The only collective is the timing reduction
(max over ranks) of a benchmark.
"""
from __future__ import annotations

from typing import Sequence


def shard_replicas(sizes: Sequence[int], world: int) -> list[list[int]]:
    """Partition replica indices into `world` shares of near-equal particle count.

    Longest-processing-time greedy: replicas in decreasing size (ties by index)
    go to the currently lightest share (ties by rank). Deterministic, so every
    rank computes the same partition without communicating. Each share keeps
    ascending replica order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    loads = [0] * world
    shares: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        shares[r].append(i)
        loads[r] += int(sizes[i])
    return [sorted(s) for s in shares]


def my_replicas(sizes: Sequence[int], rank: int, world: int) -> list[int]:
    """The replica indices rank `rank` of `world` runs."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return shard_replicas(sizes, world)[rank]


def max_over_ranks(value: float, dist=None) -> float:
    """Max of a per-rank timing over all ranks (the slowest rank sets the job time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
