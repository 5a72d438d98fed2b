"""An independent check of the oracle's polygon fill: even-odd coverage of
pixel centres by brute force.

burn_polygon (rust/src/rasterization/burners.rs:261-320) pairs each row's
sorted crossings and fills [floor(x1 + 0.5), floor(x2 + 0.5)).  Pixel x of a
row is therefore covered exactly when an odd number of the row's crossings
lie strictly left of its centre x + 0.5, since floor(c + 0.5) <= x iff
c < x + 0.5.  The crossings use the reference's FP64 sequence (PolyEdge::new
and intersect_at, rust/src/geo/edges.rs:27-55, no FMA): numpy evaluates
it the same way.  This is a different algorithm from the oracle's scanline,
so the `count` rasters must agree pixel for pixel.  CPU only."""

import math

import numpy as np
import pytest

from rusterize_gb300 import synth

from _util import oracle_burn


def _brute_count(table, grid):
    nrows, ncols = grid["nrows"], grid["ncols"]
    out = np.zeros((nrows, ncols), dtype=np.int64)
    centres = np.arange(ncols, dtype=np.float64) + 0.5
    for gi in range(table.n_geoms):
        rows: dict[int, list[float]] = {}
        for p in range(int(table.part_offsets[gi]), int(table.part_offsets[gi + 1])):
            for r in range(int(table.ring_offsets[p]), int(table.ring_offsets[p + 1])):
                v0, v1 = int(table.vertex_offsets[r]), int(table.vertex_offsets[r + 1])
                px = (table.xy[v0:v1, 0] - grid["xmin"]) / grid["xres"]
                py = (grid["ymax"] - table.xy[v0:v1, 1]) / grid["yres"]
                for k in range(v1 - v0 - 1):
                    (xa, ya), (xb, yb) = (px[k], py[k]), (px[k + 1], py[k + 1])
                    if abs(ya - yb) < np.finfo(np.float64).eps:  # edges.rs:100
                        continue
                    (xt, yt), (xbo, ybo) = ((xa, ya), (xb, yb)) if ya < yb else ((xb, yb), (xa, ya))
                    dxdy = (xbo - xt) / (ybo - yt)
                    ys = min(max(math.ceil(yt - 0.5), 0), nrows)
                    ye = min(max(math.ceil(ybo - 0.5), 0), nrows)
                    for row in range(ys, ye):
                        rows.setdefault(row, []).append(xt + ((row + 0.5) - yt) * dxdy)
        for row, xs in rows.items():
            xs = np.sort(np.array(xs))
            if len(xs) % 2:  # chunks_exact(2) drops the largest crossing of an odd row
                xs = xs[:-1]
            left = np.searchsorted(xs, centres, side="left")  # crossings strictly left of each centre
            out[row] += (left % 2).astype(np.int64)
    return out


@pytest.mark.parametrize("seed", range(6))
def test_polygon_fill_is_even_odd_at_pixel_centres(seed):
    rng = np.random.default_rng(100 + seed)
    n = 25
    side = (140, 190)
    res = (float(rng.uniform(0.3, 1.7)), float(rng.uniform(0.3, 1.7)))
    x0, y0 = float(rng.uniform(-500, 500)), float(rng.uniform(-500, 500))
    w, h = side[1] * res[0], side[0] * res[1]
    t = synth.star_polygons(rng, n, (3, 60), rng.uniform(2, 0.4 * min(w, h), n), x0 + rng.uniform(-0.1 * w, 1.1 * w, n),
                            y0 + rng.uniform(-0.1 * h, 1.1 * h, n), n_holes=rng.integers(0, 3, n))
    grid = dict(nrows=side[0], ncols=side[1], xmin=x0, xmax=x0 + w, ymin=y0, ymax=y0 + h, xres=res[0], yres=res[1])
    got = oracle_burn(t, grid, fn="count", background=0, dtype="uint32")[0].astype(np.int64)
    want = _brute_count(t, grid)
    assert want.sum() > 1000 and want.max() > 1  # covered pixels, and overlaps
    assert np.array_equal(got, want), f"{int((got != want).sum())} pixels differ"
