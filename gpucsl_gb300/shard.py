"""Replicas across GPUs: independent skeleton instances split over ranks.

Skeleton solves of different instances share nothing, so the batched and serving
workloads scale out over GPUs without a collective: every rank solves its own share.
The split balances the device work (the reference's own multi-GPU entry point,
gaussian_device_manager.py:195-227, partitions the rows of ONE skeleton instead; that
single-instance split is not built here).
"""
from __future__ import annotations

import heapq


def gaussian_cost(p: int, n: int) -> float:
    """Relative device work of a Gaussian instance: the correlation product (n p^2) plus
    the level tests (about p^2 per level, far smaller for n >> 1)."""
    return float(n) * p * p + 64.0 * p * p


def discrete_cost(p: int, n: int) -> float:
    """Relative device work of a discrete instance: each of the ~p^2/2 level-0 tests scans
    2 n codes, and the higher levels scan (l + 2) n per test."""
    return 4.0 * n * p * p


def balanced_shards(costs, world: int) -> list[list[int]]:
    """Indices of `costs` split over `world` ranks by longest-processing-time-first
    (largest cost to the least loaded rank; ties to the lower rank, then the lower
    index), each rank's list ascending.  Deterministic, so every rank computes the same
    split without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + float(costs[k]), r))
    return [sorted(s) for s in out]


def my_shard(costs, world: int, rank: int) -> list[int]:
    return balanced_shards(costs, world)[rank]
