"""Multi-GPU use without a data-path collective.

A single block-tridiagonal system runs on one GPU; several GPUs serve
independent systems (many-system batches, request streams) or run replicas
of the same workload.  This module holds the host-side pieces of that: the
rank environment of a ``torch.distributed`` launch, a size-balanced
assignment of independent systems to ranks, and the max-over-ranks timing
reduction (the only collective, outside the data path).  It works with the
NCCL backend on GPUs and with gloo on CPU processes (which is how it is
tested).
"""
from __future__ import annotations

import heapq
import os


def rank_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from a torchrun-style environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def system_cost(N: int, n: int, k: int = 1) -> float:
    """Work of one system for balancing: the factorization's N n^3 plus the
    solves' N n^2 k (both up to constants shared by every system)."""
    return float(N) * n ** 3 + 6.0 * N * n * n * k


def shard_systems(costs, world: int) -> list[list[int]]:
    """Longest-processing-time assignment of independent systems to `world`
    ranks: systems in decreasing cost (ties by index), each to the rank with
    the least work so far (ties by rank).  Deterministic; every system goes to
    exactly one rank; the largest rank load is at most 4/3 of the optimum."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    shards = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    for sh in shards:
        sh.sort()
    return shards


def my_systems(costs, rank: int, world: int) -> list[int]:
    return shard_systems(costs, world)[rank]


def reduce_max(value: float) -> float:
    """Max of `value` over all ranks (identity without an initialised process
    group).  Uses a CUDA tensor under NCCL and a CPU tensor otherwise."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
