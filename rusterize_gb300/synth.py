"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is used: the reference's own benchmarks download real
vector data at run time (python/benchmarks/benchmark_rusterize.py:11-31),
which is not available offline.  All generators use numpy PCG64 and f64
world coordinates with y up; raster extent (0, 0, W, H) at resolution 1.

Star-shaped polygon: n vertex angles sorted from U[0, 2pi), vertex radius
R * U[0.4, 1.0], ring closed.  Holes (chosen here): radius R * U[0.1, 0.3],
centre offset R * U[-0.25, 0.25] per axis, 8..64 vertices.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .geometry import LINE, POINT, POLYGON, GeometryTable


@dataclass
class Workload:
    name: str
    table: GeometryTable
    values: np.ndarray | None
    extent: tuple
    res: tuple
    fn: str
    dtype: str
    background: float
    bands: np.ndarray | None = None
    n_bands: int = 1
    meta: dict = field(default_factory=dict)


def _rings(rng, centres_x, centres_y, radii, counts):
    """Vertices of closed star rings, one per entry; returns (xy, ring_sizes)."""
    counts = np.asarray(counts, dtype=np.int64)
    nr = len(counts)
    total = int(counts.sum())
    ring_id = np.repeat(np.arange(nr), counts)
    ang = rng.uniform(0.0, 2 * np.pi, total)
    order = np.lexsort((ang, ring_id))
    ang = ang[order]
    rad = np.repeat(radii, counts) * rng.uniform(0.4, 1.0, total)
    x = np.repeat(centres_x, counts) + rad * np.cos(ang)
    y = np.repeat(centres_y, counts) + rad * np.sin(ang)
    # closing vertex: after each ring's last vertex, repeat its first
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    sizes = counts + 1
    out_starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    xy = np.empty((total + nr, 2))
    dst = np.arange(total) + np.repeat(out_starts - starts, counts)
    xy[dst, 0] = x
    xy[dst, 1] = y
    xy[out_starts + counts, 0] = x[starts]
    xy[out_starts + counts, 1] = y[starts]
    return xy, sizes


def star_polygons_sorted(rng, nv, radius, cx, cy) -> GeometryTable:
    """Hole-free star polygons, one per entry of the arrays nv (vertex
    counts), radius and centres, generated without sorting: the n sorted
    angles of a ring are 2 pi S_k / S_{n+1}, k = 1..n, with S the partial
    sums of n + 1 standard exponentials -- which has the law of n sorted
    U[0, 2 pi) draws.  Vertex radius R * U[0.4, 1.0]; each ring is closed."""
    nv = np.asarray(nv, dtype=np.int64)
    n = len(nv)
    k1 = nv + 1                                  # exponentials per ring
    e = rng.standard_exponential(int(k1.sum()))
    c = np.cumsum(e)
    ends = np.cumsum(k1) - 1                     # index of each ring's last exponential
    starts = ends - nv                           # index of its first
    base = np.where(starts > 0, c[np.maximum(starts - 1, 0)], 0.0)
    ring_of = np.repeat(np.arange(n), nv)
    # positions of the n partial sums S_1..S_n of every ring (its last one is the normaliser)
    pos = np.arange(int(k1.sum()))
    keep = np.ones(len(pos), dtype=bool)
    keep[ends] = False
    sums = c[keep] - base[ring_of]
    tot = (c[ends] - base)[ring_of]
    ang = 2.0 * np.pi * (sums / tot)
    rad = np.repeat(np.asarray(radius, dtype=np.float64), nv) * rng.uniform(0.4, 1.0, int(nv.sum()))
    x = np.repeat(np.asarray(cx, dtype=np.float64), nv) + rad * np.cos(ang)
    y = np.repeat(np.asarray(cy, dtype=np.float64), nv) + rad * np.sin(ang)
    out_starts = np.concatenate([[0], np.cumsum(k1)[:-1]])
    xy = np.empty((int(k1.sum()), 2))
    dst = np.arange(int(nv.sum())) + np.repeat(out_starts - np.concatenate([[0], np.cumsum(nv)[:-1]]), nv)
    xy[dst, 0] = x
    xy[dst, 1] = y
    first = out_starts
    xy[out_starts + nv] = xy[first]              # closing vertex
    vo = np.concatenate([[0], np.cumsum(k1)]).astype(np.uint64)
    ar = np.arange(n + 1, dtype=np.uint64)
    return GeometryTable(ar, np.full(n, POLYGON, np.uint8), ar, vo, np.zeros(n, np.uint8), xy)


def star_polygons(rng, n, nv_range, radius, cx, cy, n_holes=None, hole_nv=(8, 64)) -> GeometryTable:
    """n polygons (one part each) with optional holes."""
    nv = rng.integers(nv_range[0], nv_range[1] + 1, n)
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), (n,))
    if n_holes is None:
        n_holes = np.zeros(n, dtype=np.int64)
    n_holes = np.asarray(n_holes, dtype=np.int64)
    rings_per_poly = 1 + n_holes
    R = int(rings_per_poly.sum())
    poly_of_ring = np.repeat(np.arange(n), rings_per_poly)
    first_ring = np.concatenate([[0], np.cumsum(rings_per_poly)[:-1]])
    is_hole = np.ones(R, dtype=bool)
    is_hole[first_ring] = False
    counts = np.empty(R, dtype=np.int64)
    counts[first_ring] = nv
    nh = int(is_hole.sum())
    counts[is_hole] = rng.integers(hole_nv[0], hole_nv[1] + 1, nh)
    rr = radius[poly_of_ring].copy()
    ccx = np.asarray(cx, dtype=np.float64)[poly_of_ring].copy()
    ccy = np.asarray(cy, dtype=np.float64)[poly_of_ring].copy()
    rh = rr[is_hole]
    rr[is_hole] = rh * rng.uniform(0.1, 0.3, nh)
    ccx[is_hole] += rh * rng.uniform(-0.25, 0.25, nh)
    ccy[is_hole] += rh * rng.uniform(-0.25, 0.25, nh)
    xy, sizes = _rings(rng, ccx, ccy, rr, counts)
    vertex_offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    ring_offsets = np.concatenate([[0], np.cumsum(rings_per_poly)]).astype(np.uint64)
    return GeometryTable(np.arange(n + 1, dtype=np.uint64), np.full(n, POLYGON, np.uint8), ring_offsets,
                         vertex_offsets, is_hole.astype(np.uint8), xy)


def random_walk_lines(rng, n, nv_range, step_range, extent) -> GeometryTable:
    nv = rng.integers(nv_range[0], nv_range[1] + 1, n)
    total = int(nv.sum())
    start_x = rng.uniform(extent[0], extent[2], n)
    start_y = rng.uniform(extent[1], extent[3], n)
    step = rng.uniform(step_range[0], step_range[1], total)
    head = rng.uniform(0, 2 * np.pi, total)
    dx, dy = step * np.cos(head), step * np.sin(head)
    starts = np.concatenate([[0], np.cumsum(nv)[:-1]])
    dx[starts] = 0.0
    dy[starts] = 0.0
    line_id = np.repeat(np.arange(n), nv)
    cx = np.cumsum(dx)
    cy = np.cumsum(dy)
    cx -= np.repeat(cx[starts], nv)
    cy -= np.repeat(cy[starts], nv)
    xy = np.stack([cx + start_x[line_id], cy + start_y[line_id]], axis=1)
    vo = np.concatenate([[0], np.cumsum(nv)]).astype(np.uint64)
    return GeometryTable(np.arange(n + 1, dtype=np.uint64), np.full(n, LINE, np.uint8),
                         np.arange(n + 1, dtype=np.uint64), vo, np.zeros(n, np.uint8), xy)


def random_points(rng, n, extent) -> GeometryTable:
    xy = np.stack([rng.uniform(extent[0], extent[2], n), rng.uniform(extent[1], extent[3], n)], axis=1)
    ar = np.arange(n + 1, dtype=np.uint64)
    return GeometryTable(ar, np.full(n, POINT, np.uint8), ar, ar, np.zeros(n, np.uint8), xy)


def plain_small(seed: int = 1001) -> Workload:
    """1,000 star polygons (8-64 vertices, R ~ U[5, 50], centres U[0,1000]^2),
    f64 values U[0,100), 1000x1000 raster at resolution 1, 'last', f64, NaN bg."""
    rng = np.random.default_rng(seed)
    n = 1000
    cx, cy = rng.uniform(0, 1000, n), rng.uniform(0, 1000, n)
    radius = rng.uniform(5, 50, n)
    t = star_polygons(rng, n, (8, 64), radius, cx, cy)
    values = rng.uniform(0, 100, n)
    return Workload("plain_1k_polygons_1000x1000", t, values, (0.0, 0.0, 1000.0, 1000.0), (1.0, 1.0), "last",
                    "float64", float("nan"))


def large_fill(seed: int = 1002, scale: float = 1.0, fn: str = "sum") -> Workload:
    """100,000 polygons with 0-3 holes (outer 16-512 vertices, holes 8-64),
    radius lognormal(median 20 px, sigma_ln 1) clipped to [2, 2000], over a
    20,000 x 20,000 raster at resolution 1; f64 values U[0,1).  'sum' runs in
    float64 (NaN background), 'count' in uint32 (background 0).  `scale` < 1
    shrinks the polygon count and the raster side together (for tests)."""
    rng = np.random.default_rng(seed)
    n = max(1, int(round(100_000 * scale)))
    side = max(64.0, round(20_000 * np.sqrt(scale)))
    cx, cy = rng.uniform(0, side, n), rng.uniform(0, side, n)
    radius = np.clip(np.exp(np.log(20.0) + rng.normal(0, 1.0, n)), 2.0, 2000.0)
    holes = rng.integers(0, 4, n)
    t = star_polygons(rng, n, (16, 512), radius, cx, cy, n_holes=holes)
    values = rng.uniform(0, 1, n)
    if fn == "count":
        return Workload(f"large_fill_count_{int(side)}", t, None, (0.0, 0.0, side, side), (1.0, 1.0), "count",
                        "uint32", 0.0)
    return Workload(f"large_fill_sum_{int(side)}", t, values, (0.0, 0.0, side, side), (1.0, 1.0), "sum",
                    "float64", float("nan"))


def mixed(seed: int = 1003, scale: float = 1.0) -> tuple[Workload, Workload]:
    """50,000 polygons (large_fill generator) + 200,000 random-walk linestrings
    (2-200 vertices, steps U[1, 20] px) + 1,000,000 points over 40,000^2.
    Category U{0..15} per geometry: (i) by=str(category) -> 16 uint8 bands,
    'any', bg 0; (ii) one int32 band, 'max' of the category, bg 0."""
    rng = np.random.default_rng(seed)
    side = max(64.0, round(40_000 * np.sqrt(scale)))
    npoly, nline, npt = (max(1, int(round(k * scale))) for k in (50_000, 200_000, 1_000_000))
    ext = (0.0, 0.0, side, side)
    cx, cy = rng.uniform(0, side, npoly), rng.uniform(0, side, npoly)
    radius = np.clip(np.exp(np.log(20.0) + rng.normal(0, 1.0, npoly)), 2.0, 2000.0)
    polys = star_polygons(rng, npoly, (16, 512), radius, cx, cy, n_holes=rng.integers(0, 4, npoly))
    lines = random_walk_lines(rng, nline, (2, 200), (1.0, 20.0), ext)
    pts = random_points(rng, npt, ext)
    t = GeometryTable.concat([polys, lines, pts])
    cat = rng.integers(0, 16, t.n_geoms)
    names = sorted({str(c) for c in range(16)})  # BTreeMap order of the string keys
    band_of = {k: i for i, k in enumerate(names)}
    bands = np.array([band_of[str(c)] for c in cat], dtype=np.uint32)
    a = Workload(f"mixed_any_16band_{int(side)}", t, None, ext, (1.0, 1.0), "any", "uint8", 0.0, bands, 16,
                 {"band_names": names})
    b = Workload(f"mixed_max_int32_{int(side)}", t, cat.astype(np.int32), ext, (1.0, 1.0), "max", "int32", 0.0)
    return a, b


BATCH_FNS = ("sum", "min", "max", "first", "last", "count")


def batch_jobs_fast(seed: int = 1004, n_jobs: int = 4096, side_range: tuple = (256.0, 8192.0),
                    max_polygons: int = 50_000, chunk: int = 128, threads: int | None = None) -> list[Workload]:
    """The batch_jobs distributions, generated many jobs at a time: chunks of
    `chunk` jobs, each from its own stream of SeedSequence(seed) (so the
    result does not depend on `threads`), built on host threads with
    star_polygons_sorted over the chunk and split per job.  Same parameters
    and laws as batch_jobs; different draws, so the jobs differ from
    batch_jobs(seed)'s."""
    import concurrent.futures as cf
    import os

    lo, hi = np.log(side_range[0]), np.log(side_range[1])
    n_chunks = (n_jobs + chunk - 1) // chunk
    seeds = np.random.SeedSequence(seed).spawn(max(1, n_chunks))

    def make(ci: int) -> list[Workload]:
        rng = np.random.default_rng(seeds[ci])
        c0 = ci * chunk
        m = min(chunk, n_jobs - c0)
        npoly = np.clip(np.round(np.exp(np.log(500.0) + rng.normal(0.0, 1.0, m))), 10, max_polygons).astype(np.int64)
        side = np.round(np.exp(rng.uniform(lo, hi, m)))
        fns = rng.integers(0, len(BATCH_FNS), m)
        job_of = np.repeat(np.arange(m), npoly)
        s_of = side[job_of]
        radius = np.clip(np.exp(np.log(0.02 * s_of) + rng.normal(0.0, 1.0, len(job_of))), 2.0, 0.25 * s_of)
        cx, cy = rng.uniform(0.0, 1.0, len(job_of)) * s_of, rng.uniform(0.0, 1.0, len(job_of)) * s_of
        nv = rng.integers(8, 257, len(job_of))
        t = star_polygons_sorted(rng, nv, radius, cx, cy)
        values = rng.uniform(0, 1, len(job_of)).astype(np.float32)
        g = np.concatenate([[0], np.cumsum(npoly)])
        out = []
        for j in range(m):
            sd = float(side[j])
            out.append(Workload(f"batch_job_{c0 + j}", t.slice(int(g[j]), int(g[j + 1])),
                                values[g[j]:g[j + 1]].copy(), (0.0, 0.0, sd, sd), (1.0, 1.0), BATCH_FNS[int(fns[j])],
                                "float32", float("nan")))
        return out

    nt = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max(1, nt)) as ex:
        parts = list(ex.map(make, range(n_chunks)))
    return [w for p in parts for w in p]


def batch_jobs(seed: int = 1004, n_jobs: int = 4096, side_range: tuple = (256.0, 8192.0),
               max_polygons: int = 50_000) -> list[Workload]:
    """Independent jobs of uneven size: polygons per job lognormal (median
    500, sigma_ln 1) clipped to [10, max_polygons], 8-256 vertices each; raster
    side log-uniform over `side_range` at resolution 1; radius lognormal
    (median 0.02 side, sigma_ln 1) clipped to [2, 0.25 side]; f32 values
    U[0, 1); pixel function uniform over BATCH_FNS; float32 output, NaN
    background."""
    rng = np.random.default_rng(seed)
    jobs = []
    lo, hi = np.log(side_range[0]), np.log(side_range[1])
    for j in range(n_jobs):
        n = int(np.clip(round(float(np.exp(np.log(500.0) + rng.normal(0.0, 1.0)))), 10, max_polygons))
        side = float(round(float(np.exp(rng.uniform(lo, hi)))))
        radius = np.clip(np.exp(np.log(0.02 * side) + rng.normal(0.0, 1.0, n)), 2.0, 0.25 * side)
        cx, cy = rng.uniform(0, side, n), rng.uniform(0, side, n)
        t = star_polygons(rng, n, (8, 256), radius, cx, cy)
        values = rng.uniform(0, 1, n).astype(np.float32)
        fn = BATCH_FNS[int(rng.integers(0, len(BATCH_FNS)))]
        jobs.append(Workload(f"batch_job_{j}", t, values, (0.0, 0.0, side, side), (1.0, 1.0), fn, "float32",
                             float("nan")))
    return jobs
