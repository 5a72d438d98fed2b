"""Spreading independent burn jobs over the GPUs of one node.

The burn path has no exchange step: jobs (and the bands or rows of one job)
are independent, so N GPUs run N disjoint shares with no collective on the
data path.  The only collectives are for timing and reporting: the step time
of a multi-GPU run is the slowest rank's, and its work the sum of all
ranks'.  One process drives one GPU; ranks come from the usual torchrun
environment (RANK, WORLD_SIZE, LOCAL_RANK).
"""

from __future__ import annotations

import heapq
import os
from collections.abc import Sequence


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard_jobs(costs: Sequence[float], world: int) -> list[list[int]]:
    """Balanced shares of jobs with the given costs (e.g. raster pixels plus
    vertices): longest job first to the least loaded rank, ties to the lower
    rank.  Deterministic, so every rank computes the same shares.  Each
    share lists its jobs in their original order."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    heap = [(0.0, r) for r in range(world)]
    shares: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def job_cost(nrows: int, ncols: int, n_vertices: int) -> float:
    """Cost model of one job: its raster is written once, and its vertices
    drive the coverage work."""
    return float(nrows) * float(ncols) + 32.0 * float(n_vertices)


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (a step time); the value itself on
    one rank or without an initialised process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    """The sum over all ranks (units of work)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
