"""Replicas across GPUs: independent systems, no data-path collective.

Ensembles and served requests shard by system (each system's state, noise and
neighbour sums are its own), so N ranks run N independent batches.  This module
holds the host logic: a deterministic footprint-balanced partition of the
systems over the ranks, and the two reductions the measurement needs (the
slowest rank's time, the total work).  With torch.distributed it works over
NCCL on GPUs and over gloo on the CPU (the tests).
"""
from __future__ import annotations

import heapq
from typing import Optional, Sequence


def partition_by_footprint(sizes: Sequence[int], world: int) -> list[list[int]]:
    """Indices of the systems each rank runs.

    Longest-processing-time order: systems by decreasing size (ties by index),
    each to the rank with the smallest load so far (ties by rank).  Every
    system lands on exactly one rank; the largest load exceeds the mean by at
    most the largest system.  Within a rank the indices are ascending."""
    if world <= 0:
        raise ValueError("world must be positive")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(v) for v in out]


def shard(sizes: Sequence[int], world: int, rank: int) -> list[int]:
    """The systems of one rank."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return partition_by_footprint(sizes, world)[rank]


def max_over_ranks(value: float, dist=None, device: Optional[str] = None) -> float:
    """The largest value over all ranks (the job's time is the slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device: Optional[str] = None) -> float:
    """The total over all ranks (work done by the whole job)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
