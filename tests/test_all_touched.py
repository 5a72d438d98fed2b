"""all_touched on the GPU vs the oracle (AllTouched::burn_line,
rust/src/rasterization/burners.rs:94-247; polygon rings walked before the
fill, burn_geometry.rs:76-166, 212-243; PixelCache for sum / count,
prelude.rs:116-118 and pixel_cache.rs), bit-exact, through the C ABI."""

import zlib

import numpy as np
import pytest

from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth

from _util import diff_report, gpu_burn, oracle_burn, same_bits

pytestmark = pytest.mark.gpu

FNS = ["sum", "first", "last", "min", "max", "count", "any"]


def check(table, grid, **kw):
    got = gpu_burn(table, grid, all_touched=True, **kw)
    ref = oracle_burn(table, grid, all_touched=True, **kw)
    assert same_bits(got, ref), diff_report(got, ref)
    return got


def _grid(n, m=None, res=(1.0, 1.0), x0=0.0, y0=0.0):
    m = n if m is None else m
    return dict(nrows=n, ncols=m, xmin=x0, xmax=x0 + m * res[0], ymin=y0, ymax=y0 + n * res[1], xres=res[0],
                yres=res[1])


def test_diagonal_line_touches_more_cells_than_centre_sampling():
    # R/rusterize/tests/testthat/test-geometry.R:25-30
    b = G.TableBuilder()
    G.add_linestring(b, [(0, 0), (4, 4)])
    t = b.build()
    grid = _grid(4)
    off = gpu_burn(t, grid, fn="last", values=np.array([9.0]), background=0.0)
    on = check(t, grid, fn="last", values=np.array([9.0]), background=0.0)
    assert (on > 0).sum() > (off > 0).sum()


@pytest.mark.parametrize("fn", FNS)
def test_polygons_lines_points_every_function(fn):
    rng = np.random.default_rng(zlib.crc32(fn.encode()))
    side = 120
    n = 150
    polys = synth.star_polygons(rng, n, (3, 30), rng.uniform(1.0, 25.0, n), rng.uniform(-20, side + 20, n),
                                rng.uniform(-20, side + 20, n), n_holes=rng.integers(0, 3, n))
    lines = synth.random_walk_lines(rng, 80, (2, 30), (0.3, 12.0), (-10, -10, side + 10, side + 10))
    pts = synth.random_points(rng, 60, (0, 0, side, side))
    t = G.GeometryTable.concat([polys, lines, pts])
    v = rng.integers(1, 6, t.n_geoms).astype(np.float64)
    for bg in (0.0, np.nan, 3.0):
        check(t, _grid(side), fn=fn, values=v, background=bg, dtype="float64")


@pytest.mark.parametrize("res", [(1.0, 1.0), (0.5, 0.5), (1.0, 0.75), (0.37, 0.61)])
def test_resolutions_sum_and_count(res):
    rng = np.random.default_rng(31)
    n = 120
    side = 60.0
    polys = synth.star_polygons(rng, n, (3, 24), rng.uniform(0.5, 10.0, n), rng.uniform(-5, side + 5, n),
                                rng.uniform(-5, side + 5, n), n_holes=rng.integers(0, 2, n))
    lines = synth.random_walk_lines(rng, 60, (2, 20), (0.2, 6.0), (0, 0, side, side))
    t = G.GeometryTable.concat([polys, lines])
    nrows, ncols = int(side / res[1]), int(side / res[0])
    grid = dict(nrows=nrows, ncols=ncols, xmin=0.0, xmax=ncols * res[0], ymin=0.0, ymax=nrows * res[1],
                xres=res[0], yres=res[1])
    v = rng.integers(1, 4, t.n_geoms).astype(np.int32)
    for fn in ("sum", "count", "last"):
        check(t, grid, fn=fn, values=v, background=0, dtype="int32")
    check(t, grid, fn="count", values=None, background=0, dtype="uint16")


def test_axis_aligned_and_degenerate_segments():
    b = G.TableBuilder()
    G.add_linestring(b, [(2.0, 1.0), (2.005, 8.5)])       # nearly vertical
    G.add_linestring(b, [(1.0, 3.0), (9.5, 3.004)])       # nearly horizontal
    G.add_linestring(b, [(0.0, 0.0), (10.0, 10.0)])       # exact diagonal through corners
    G.add_linestring(b, [(3.0, 9.0), (7.0, 1.0), (3.0, 9.0)])
    G.add_linestring(b, [(-5.0, 4.5), (15.0, 5.5)])       # clipped on both sides
    G.add_linestring(b, [(4.0, -3.0), (6.0, 13.0)])       # clipped top and bottom
    G.add_polygon(b, np.array([[1.0, 1.0], [9.0, 1.0], [9.0, 9.0], [1.0, 9.0], [1.0, 1.0]]))
    G.add_polygon(b, np.array([[4.5, 4.5], [5.5, 4.5], [5.5, 5.5], [4.5, 5.5], [4.5, 4.5]]))
    t = b.build()
    grid = _grid(10)
    v = np.arange(1, t.n_geoms + 1, dtype=np.float64)
    for fn in FNS:
        check(t, grid, fn=fn, values=v, background=0.0)


def test_polygons_crossing_every_border():
    # rings that leave the raster on each side (edges outside it are dropped
    # from the walk by extract_line's filter)
    rng = np.random.default_rng(77)
    n = 200
    side = 80
    cx = np.concatenate([rng.uniform(-15, 5, n // 4), rng.uniform(side - 5, side + 15, n // 4),
                         rng.uniform(0, side, n // 2)])
    cy = np.concatenate([rng.uniform(0, side, n // 2), rng.uniform(-15, 5, n // 4),
                         rng.uniform(side - 5, side + 15, n // 4)])
    polys = synth.star_polygons(rng, n, (3, 20), rng.uniform(2.0, 30.0, n), cx, cy, n_holes=rng.integers(0, 2, n))
    v = rng.integers(1, 5, n).astype(np.float64)
    for fn in ("sum", "count", "last", "min"):
        check(polys, _grid(side), fn=fn, values=v, background=0.0)


def test_bands_and_large_raster():
    a, _ = synth.mixed(scale=0.0005)
    from rusterize_gb300.engine import raster_info

    info = raster_info(a.table, res=a.res, extent=a.extent)
    grid = dict(nrows=info.nrows, ncols=info.ncols, xmin=info.xmin, xmax=info.xmax, ymin=info.ymin, ymax=info.ymax,
                xres=info.xres, yres=info.yres)
    check(a.table, grid, fn="any", values=None, background=0, dtype="uint8", bands=a.bands, n_bands=a.n_bands)
    check(a.table, grid, fn="sum", values=None, background=0, dtype="uint16", bands=a.bands, n_bands=a.n_bands)
