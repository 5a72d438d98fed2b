"""Spreading burn work over the GPUs of one node.

The burn path has no exchange step: jobs, and the bands or rows of one job,
are independent, so N GPUs run N disjoint shares with no collective on the
data path.  Two splits:

* independent jobs (``shard_jobs``): each rank burns whole jobs;
* the rows of one job (``row_bands``, ``select_rows``): rank k burns the
  raster rows [r_k, r_k+1) of the same job with ``rz_rasterize_rows``, from
  the geometries that can write there, in input order, and writes a
  disjoint slice of the raster.  Every pixel decision is taken on the whole
  raster's grid, so the slices put together equal the whole burn.

The only collectives are for timing and reporting: the step time of a
multi-GPU run is the slowest rank's, and its work the sum of all ranks'.
One process drives one GPU; ranks come from the usual torchrun environment
(RANK, WORLD_SIZE, LOCAL_RANK).
"""

from __future__ import annotations

import heapq
import os
from collections.abc import Sequence

import numpy as np


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


def row_bands(nrows: int, world: int, row_cost: Sequence[float] | None = None) -> list[tuple[int, int]]:
    """Contiguous row bands [r0, r1), one per rank, that cover rows [0, nrows)
    once, in order.  With `row_cost` (one non-negative cost per row, e.g. the
    pixel writes expected in it) the bands balance the cost; otherwise they
    balance the rows.  Deterministic, so every rank computes the same bands."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    if row_cost is None:
        edges = [nrows * k // world for k in range(world + 1)]
    else:
        c = np.asarray(row_cost, dtype=np.float64)
        if c.shape != (nrows,) or (c < 0).any():
            raise ValueError("row_cost needs one non-negative cost per row")
        cum = np.concatenate([[0.0], np.cumsum(c)])
        total = cum[-1]
        edges = [0]
        for k in range(1, world):
            # first row boundary whose cumulative cost reaches k / world of the total
            e = int(np.searchsorted(cum, total * k / world, side="left")) if total > 0 else nrows * k // world
            edges.append(min(max(e, edges[-1]), nrows))
        edges.append(nrows)
    return [(int(edges[k]), int(edges[k + 1])) for k in range(world)]


def geometry_rows(table, info) -> tuple[np.ndarray, np.ndarray]:
    """A conservative range [lo, hi] of raster rows each geometry can write.

    Every pixel a geometry burns lies within one row of the pixel rows of its
    vertices: polygon scanlines run between ceil(y - 0.5) of its extreme
    vertices, Bresenham and AllTouched walks between floor(y) of a
    segment's end points (AllTouched nudges y by 1e-9 at most), and a point
    is floor(y).  A geometry with a non-finite coordinate, or none, gets the
    whole raster, so no selection can drop a write."""
    G = table.n_geoms
    po = table.part_offsets.astype(np.int64)
    ro = table.ring_offsets.astype(np.int64)
    vo = table.vertex_offsets.astype(np.int64)
    v_start = vo[ro[po[:-1]]]  # first vertex of each geometry
    v_end = vo[ro[po[1:]]]
    y = table.xy[:, 1]
    py = (info.ymax - y) / info.yres
    lo = np.full(G, 0, dtype=np.int64)
    hi = np.full(G, info.nrows - 1, dtype=np.int64)
    has = v_end > v_start
    if has.any() and len(py):
        starts = v_start[has]
        with np.errstate(invalid="ignore"):
            mn = np.minimum.reduceat(py, starts)
            mx = np.maximum.reduceat(py, starts)
            bad = np.logical_or.reduceat(~np.isfinite(py), starts)
        ok = ~bad & np.isfinite(mn) & np.isfinite(mx)
        idx = np.nonzero(has)[0]
        lo_v = np.floor(mn[ok]) - 1
        hi_v = np.floor(mx[ok]) + 1
        lo[idx[ok]] = np.clip(lo_v, -1, info.nrows).astype(np.int64)
        hi[idx[ok]] = np.clip(hi_v, -1, info.nrows).astype(np.int64)
    return lo, hi


def select_rows(table, info, r0: int, r1: int) -> np.ndarray:
    """Indices (ascending: input order) of the geometries that can write a
    pixel in rows [r0, r1).  The others write nothing there, so burning the
    selection into that window gives the window of the whole burn."""
    lo, hi = geometry_rows(table, info)
    return np.nonzero((hi >= r0) & (lo < r1))[0]


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
