"""The oracle's sparse stream (SparseArrayWriter, rust/src/encoding/
writers.rs:86-131) replayed the way SparseArray::build_array does it
(rust/src/encoding/arrays.rs:103-141, pixel functions of
rust/src/rasterization/pixel_functions.rs:56-122) equals the oracle's dense
raster, which is pinned to the reference's golden rasters.  CPU only."""

import numpy as np
import pytest

import oracle
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth

from _util import GOLDEN, golden_inputs, grid_of, oracle_burn, same_bits


def _apply(fn, cur, v, bg):
    nan = cur != cur
    if fn == "sum":
        return v if (cur == bg or nan or v != v) else cur + v
    if fn == "first":
        return v if (cur == bg or nan) else cur
    if fn == "last":
        return v
    if fn == "min":
        return v if (cur == bg or nan or cur > v) else cur
    if fn == "max":
        return v if (cur == bg or nan or cur < v) else cur
    if fn == "count":
        return cur.dtype.type(1) if (cur == bg or nan) else cur + cur.dtype.type(1)
    return cur.dtype.type(1)  # any


def replay(sparse, shape, fn, bg, dtype):
    band_counts, rows, cols, vals = sparse
    out = np.full(shape, bg, dtype=dtype)
    bg = np.array(bg, dtype=dtype)[()]
    i = 0
    with np.errstate(over="ignore"):
        for b, n in enumerate(band_counts.tolist()):
            for k in range(i, i + n):
                r, c = int(rows[k]), int(cols[k])
                out[b, r, c] = _apply(fn, out[b, r, c], vals[k], bg)
            i += n
    return out


def _sparse(t, grid, **kw):
    g = grid_of(grid)
    return oracle.rasterize_sparse(t, g["nrows"], g["ncols"], g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["xres"],
                                   g["yres"], **kw)


def test_golden_standard_output_sum_from_the_sparse_stream():
    # python/test/test_many.py:216-235: sparse to_numpy == numpy == the golden raster
    geoms, values = golden_inputs()
    t = G.from_wkt(geoms)
    info = oracle.raster_info(t, res=(1, 1))
    sp = _sparse(t, info, fn="sum", values=values, dtype="uint8")
    r = replay(sp, (1, info[0], info[1]), "sum", 0, np.uint8)
    assert np.array_equal(r[0], np.load(GOLDEN / "standard_output_sum.npy"))


@pytest.mark.parametrize("touched", [False, True])
@pytest.mark.parametrize("fn", ["sum", "first", "last", "min", "max", "count", "any"])
def test_replay_equals_dense(fn, touched):
    rng = np.random.default_rng(77)
    side, n = 60, 40
    polys = synth.star_polygons(rng, n, (3, 20), rng.uniform(1.0, 15.0, n), rng.uniform(-5, side + 5, n),
                                rng.uniform(-5, side + 5, n), n_holes=rng.integers(0, 2, n))
    lines = synth.random_walk_lines(rng, 20, (2, 12), (0.5, 8.0), (-5, -5, side + 5, side + 5))
    pts = synth.random_points(rng, 20, (0, 0, side, side))
    t = G.GeometryTable.concat([polys, lines, pts])
    v = rng.integers(1, 6, t.n_geoms).astype(np.float64)
    bands = rng.integers(0, 2, t.n_geoms).astype(np.uint32)
    grid = dict(nrows=side, ncols=side, xmin=0.0, xmax=float(side), ymin=0.0, ymax=float(side), xres=1.0, yres=1.0)
    for bg in (0.0, np.nan):
        sp = _sparse(t, grid, fn=fn, values=v, bands=bands, n_bands=2, all_touched=touched)
        dense = oracle_burn(t, grid, fn=fn, values=v, background=bg, bands=bands, n_bands=2, all_touched=touched)
        assert int(sp[0].sum()) == len(sp[1])
        assert same_bits(replay(sp, dense.shape, fn, bg, np.float64), dense)
