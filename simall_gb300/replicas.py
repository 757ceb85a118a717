"""Host-side logic of multi-process runs: one process per GPU.

A single pressure system is not partitioned across GPUs; N processes either
solve N independent replicas (the benchmark's headline solve) or share a batch
of independent systems (the batched solve), with no collective on the data
path.  What crosses processes is host control only: the rank layout, the
assignment of batch systems to ranks, and the maximum of the ranks' timings.
"""
from __future__ import annotations

import os

import numpy as np


def rank_info() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def shard_by_cost(costs, rank: int, world: int) -> np.ndarray:
    """Indices of the items this rank takes: longest-processing-time-first
    greedy assignment (items by decreasing cost, each to the least-loaded rank,
    ties to the lowest rank), identical on every rank without communication.
    Every item goes to exactly one rank."""
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return np.flatnonzero(owner == rank)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar over the default process group (any
    backend; `device` is where the reduction tensor lives: CPU for gloo, the
    rank's GPU for NCCL).  Without an initialised group it returns value."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
