"""GPU engine vs the oracle: bit-exact parity on the reference's golden
inputs and KATs, on seeded synthetic workloads for every pixel function and
dtype, and on edge cases.  Every call goes through the C ABI."""

import zlib

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth

from _kats import all_kats, sq
from _util import GOLDEN, diff_report, explode, golden_inputs, gpu_burn, oracle_burn, same_bits

pytestmark = pytest.mark.gpu

FNS = ["sum", "first", "last", "min", "max", "count", "any"]
DTYPES = ["uint8", "uint16", "uint32", "uint64", "int8", "int16", "int32", "int64", "float32", "float64"]


def check(table, grid, **kw):
    stats = {}
    got = gpu_burn(table, grid, stats=stats, **kw)
    ref = oracle_burn(table, grid, **kw)
    assert same_bits(got, ref), diff_report(got, ref)
    return stats


def test_golden_standard_output_sum_gpu():
    geoms, values = golden_inputs()
    t = G.from_wkt(geoms)
    info = rz.raster_info(t, res=(1, 1))
    r = gpu_burn(t, info, fn="sum", values=values, background=0, dtype="uint8")
    assert np.array_equal(r[0], np.load(GOLDEN / "standard_output_sum.npy"))


def test_golden_custom_shape_gpu():
    geoms, values = golden_inputs()
    t, v = explode(G.from_wkt(geoms), values)
    info = rz.raster_info(t, shape=(47, 319))
    r = gpu_burn(t, info, fn="sum", values=v, background=0, dtype="uint8")
    assert np.array_equal(r[0], np.load(GOLDEN / "standard_output_sum_custom_shape.npy"))


@pytest.mark.parametrize("kat", all_kats(), ids=lambda k: k[0])
def test_kats_gpu(kat):
    name, t, grid, kw, expected = kat
    r = gpu_burn(t, grid, **kw)
    if callable(expected):
        assert expected(r), name
    else:
        np.testing.assert_array_equal(r, expected)


def test_plain_small_config():
    w = synth.plain_small(1001)
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    stats = check(w.table, info, fn=w.fn, values=w.values, background=w.background, dtype=w.dtype)
    assert stats["pixel_writes"] > 1_000_000


def _random_polys(seed, n, side, rmax=30.0, holes=True):
    rng = np.random.default_rng(seed)
    cx, cy = rng.uniform(-10, side + 10, n), rng.uniform(-10, side + 10, n)
    radius = rng.uniform(1.0, rmax, n)
    nh = rng.integers(0, 3, n) if holes else None
    return synth.star_polygons(rng, n, (3, 40), radius, cx, cy, n_holes=nh)


def _values(rng, n, dtype, bg):
    dt = np.dtype(dtype)
    if dt.kind == "f":
        v = rng.integers(-3, 8, n).astype(dt)
        v[rng.random(n) < 0.05] = np.nan
    else:
        info = np.iinfo(dt)
        v = rng.integers(max(info.min, -3), min(info.max, 8) + 1, n).astype(dt)
    # some values equal to the background: exercises the reset semantics
    if not (isinstance(bg, float) and np.isnan(bg)):
        v[rng.random(n) < 0.1] = dt.type(bg)
    return v


@pytest.mark.parametrize("fn", FNS)
@pytest.mark.parametrize("dtype", ["uint8", "int16", "int64", "float32", "float64"])
def test_overlap_semantics(fn, dtype):
    rng = np.random.default_rng(zlib.crc32(f"{fn}/{dtype}".encode()))
    t = _random_polys(7, 300, 200)
    bgs = [0, 2] if np.dtype(dtype).kind != "f" else [np.nan, 0.0, 2.0]
    for bg in bgs:
        v = _values(rng, t.n_geoms, dtype, bg)
        grid = dict(nrows=200, ncols=200, xmin=0.0, xmax=200.0, ymin=0.0, ymax=200.0, xres=1.0, yres=1.0)
        check(t, grid, fn=fn, values=v, background=bg, dtype=dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_all_dtypes_sum_and_first(dtype):
    rng = np.random.default_rng(11)
    t = _random_polys(3, 200, 150)
    v = _values(rng, t.n_geoms, dtype, 0)
    grid = dict(nrows=150, ncols=150, xmin=0.0, xmax=150.0, ymin=0.0, ymax=150.0, xres=1.0, yres=1.0)
    for fn in ("sum", "first", "count"):
        check(t, grid, fn=fn, values=v, background=0, dtype=dtype)


def test_large_fill_scaled_sum_and_count():
    w = synth.large_fill(scale=0.01, fn="sum")
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    check(w.table, info, fn="sum", values=w.values, background=np.nan, dtype="float64")
    check(w.table, info, fn="count", values=None, background=0, dtype="uint32")


def test_wide_raster_tiles_and_resolution():
    # > 1024 columns (several column tiles per row), non-power-of-two resolution
    rng = np.random.default_rng(5)
    n = 400
    t = synth.star_polygons(rng, n, (8, 64), rng.uniform(2, 300, n), rng.uniform(0, 3000, n),
                            rng.uniform(0, 300, n), n_holes=rng.integers(0, 2, n))
    v = rng.uniform(0, 1, n)
    info = rz.raster_info(t, res=(0.7, 0.7))
    check(t, info, fn="sum", values=v, background=np.nan, dtype="float64")
    info2 = rz.raster_info(t, shape=(211, 2917))
    check(t, info2, fn="last", values=v, background=-1.0, dtype="float32")


def test_lines_points_and_bands():
    a, b = synth.mixed(scale=0.0005)
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    check(a.table, info, fn="any", values=None, background=0, dtype="uint8", bands=a.bands, n_bands=a.n_bands)
    check(b.table, info, fn="max", values=b.values, background=0, dtype="int32")
    check(b.table, info, fn="sum", values=b.values, background=0, dtype="int32")
    check(b.table, info, fn="count", values=None, background=0, dtype="uint16")


@pytest.mark.parametrize("fn", ["sum", "count", "last"])
def test_non_square_pixels_line_dedup(fn):
    # LineString burns through a PixelCache when xres != yres (burn_geometry.rs:179-185)
    rng = np.random.default_rng(9)
    lines = synth.random_walk_lines(rng, 300, (2, 60), (1.0, 15.0), (0, 0, 300, 300))
    info = rz.raster_info(lines, res=(1.0, 0.75))
    v = rng.integers(1, 5, lines.n_geoms).astype(np.float64)
    check(lines, info, fn=fn, values=v, background=0.0, dtype="float64")


def test_multilinestring_and_closed_rings():
    b = G.TableBuilder()
    G.add_multilinestring(b, [[(1, 1), (8, 3), (2, 7)], [(2, 7), (9, 9)], [(5, 5), (5, 5)]])
    G.add_linestring(b, [(1, 9), (9, 9), (9, 1), (1, 9)])  # closed: no end pixel
    G.add_linestring(b, [(0.5, 0.5), (12.0, 12.0)])       # leaves the raster
    G.add_linestring(b, [(-5, 3.5), (-1, 3.5)])            # entirely outside
    G.add_multipoint(b, [(1.5, 1.5), (1.5, 1.5), (20, 20), (9.99, 0.01)])
    t = b.build()
    grid = dict(nrows=10, ncols=10, xmin=0.0, xmax=10.0, ymin=0.0, ymax=10.0, xres=1.0, yres=1.0)
    for fn in FNS:
        check(t, grid, fn=fn, values=np.arange(1, t.n_geoms + 1, dtype=np.float64), background=0.0)


def test_collections_and_empty_parts():
    t = G.from_wkt([
        "GEOMETRYCOLLECTION (POINT (5 5), POLYGON ((2 2, 8 2, 8 8, 2 8, 2 2)), LINESTRING (0 0, 10 10))",
        "MULTIPOLYGON (((1 1, 5 1, 5 5, 1 5, 1 1)), ((3 3, 9 3, 9 9, 3 9, 3 3)))",
        "POLYGON EMPTY",
        "GEOMETRYCOLLECTION EMPTY",
        "LINESTRING EMPTY",
        "POLYGON ((0 0, 10 0, 10 10, 0 10, 0 0), (2 2, 4 2, 4 4, 2 4, 2 2))",
        "POLYGON ((-100 -100, 100 -100, 100 100, -100 100, -100 -100))",
    ])
    grid = dict(nrows=10, ncols=10, xmin=0.0, xmax=10.0, ymin=0.0, ymax=10.0, xres=1.0, yres=1.0)
    for fn in FNS:
        check(t, grid, fn=fn, values=np.arange(1, t.n_geoms + 1, dtype=np.int32), background=0, dtype="int32")


def test_big_buckets_ordered():
    # thousands of polygons over one 1024-column tile: the block-level path,
    # including part ranges beyond 4096 spans per bucket
    rng = np.random.default_rng(21)
    n = 6000
    t = synth.star_polygons(rng, n, (3, 12), rng.uniform(3, 30, n), rng.uniform(0, 64, n), rng.uniform(0, 64, n))
    v = rng.uniform(0, 1, n)
    grid = dict(nrows=64, ncols=64, xmin=0.0, xmax=64.0, ymin=0.0, ymax=64.0, xres=1.0, yres=1.0)
    stats = check(t, grid, fn="sum", values=v, background=np.nan, dtype="float64")
    assert stats["big_buckets"] > 0
    check(t, grid, fn="first", values=v, background=np.nan, dtype="float64")
    check(t, grid, fn="count", values=None, background=0, dtype="uint16")


@pytest.mark.parametrize("fn", ["first", "last", "min", "max"])
@pytest.mark.parametrize("dtype", ["int16", "float32", "float64"])
def test_order_free_folds_ties_and_resets(fn, dtype):
    """first / last / min / max fold without a sort unless a written value is
    the background or NaN: equal values (-0.0 and +0.0 among them) go to the
    earliest part, and a value equal to the background, or NaN, sends the tile
    back to the sorted fold.  300 polygons over 64 x 64 give tiles of a few
    hundred records (one warp per tile), 6,000 give tiles of thousands (one
    warp per word)."""
    rng = np.random.default_rng(zlib.crc32(f"of/{fn}/{dtype}".encode()))
    grid = dict(nrows=64, ncols=64, xmin=0.0, xmax=64.0, ymin=0.0, ymax=64.0, xres=1.0, yres=1.0)
    floating = np.dtype(dtype).kind == "f"
    for n in (300, 6000):
        t = synth.star_polygons(rng, n, (3, 12), rng.uniform(3, 30, n), rng.uniform(0, 64, n), rng.uniform(0, 64, n))
        for bg in ((np.nan, 0.0) if floating else (0, 3)):
            if floating:
                clean = [x for x in (0.0, -0.0, 1.0, -1.0, 2.5) if not x == bg]
                dirty = clean + [bg, np.nan]
            else:
                clean = [x for x in (0, 1, 2, 5, -1) if x != bg]
                dirty = clean + [bg]
            for pool in (clean, dirty):
                v = rng.choice(np.array(pool, dtype=dtype), n)
                stats = check(t, grid, fn=fn, values=v, background=bg, dtype=dtype)
                if n == 6000:
                    assert stats["big_buckets"] > 0


def test_single_part_many_spans_in_one_bucket():
    # one zig-zag polygon with > 4096 spans in a single row tile
    k = 5000
    xs = np.repeat(np.arange(k, dtype=np.float64) * 0.2, 2)
    ys = np.tile([0.2, 0.8], k)
    ring = np.concatenate([np.stack([xs, ys], 1), [[xs[-1], -1.0], [xs[0], -1.0], [xs[0], ys[0]]]])
    b = G.TableBuilder()
    b.add_part(G.POLYGON, [(ring, 0)])
    b.end_geometry()
    G.add_polygon(b, sq(0, 0, 1000, 1))
    t = b.build()
    grid = dict(nrows=1, ncols=1000, xmin=0.0, xmax=1000.0, ymin=0.0, ymax=1.0, xres=1.0, yres=1.0)
    for fn in ("sum", "count", "last"):
        check(t, grid, fn=fn, values=np.array([2.0, 3.0]), background=0.0)


def test_degenerate_and_nonfinite():
    b = G.TableBuilder()
    G.add_polygon(b, [(1, 1), (1, 1), (1, 1)])                  # zero area
    G.add_polygon(b, [(0, 5), (10, 5), (10, 5.0000000001)])      # near-horizontal sliver
    G.add_polygon(b, [(2, 2), (np.nan, 3), (6, 6), (2, 6)])      # NaN vertex
    G.add_polygon(b, [(0, 0.5), (10, 0.5 + 1e-17), (10, 3), (0, 3)])
    G.add_polygon(b, [(1e6, 1e6), (1e6 + 5, 1e6), (1e6, 1e6 + 5)])  # far away
    t = b.build()
    grid = dict(nrows=10, ncols=10, xmin=0.0, xmax=10.0, ymin=0.0, ymax=10.0, xres=1.0, yres=1.0)
    check(t, grid, fn="sum", values=np.arange(1.0, t.n_geoms + 1), background=0.0)


def test_span_buffer_growth_rerun():
    # steep lines give one span per pixel: > 1M spans from a few hundred
    # vertices overflow the first record buffer and force the rerun path
    rng = np.random.default_rng(4)
    b = G.TableBuilder()
    for _ in range(400):
        x0, x1 = rng.uniform(0, 4000, 2)
        G.add_linestring(b, [(x0, 0.5), (x0 + (x1 - x0) * 0.25, 3999.5)])
    t = b.build()
    grid = dict(nrows=4000, ncols=4000, xmin=0.0, xmax=4000.0, ymin=0.0, ymax=4000.0, xres=1.0, yres=1.0)
    ctx = rz.Context(0)  # fresh scratch arena
    stats = {}
    got = rz.rasterize_table(t, rz.RasterInfo(**grid), fn="count", background=0, dtype="uint8", context=ctx,
                             stats=stats)
    ref = oracle_burn(t, grid, fn="count", background=0, dtype="uint8")
    assert same_bits(got, ref), diff_report(got, ref)
    assert stats["spans"] > 1_000_000 and stats["reruns"] >= 1
    ctx.close()


def test_repeat_calls_reuse_scratch():
    w = synth.plain_small(1001)
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    first = gpu_burn(w.table, info, fn="sum", values=w.values, background=np.nan)
    for _ in range(3):
        again = gpu_burn(w.table, info, fn="sum", values=w.values, background=np.nan)
        assert same_bits(first, again)


def test_rusterize_front_end_numpy():
    geoms, values = golden_inputs()
    r = rz.rusterize(geoms, res=(1, 1), dtype="uint8", burn=values.astype(np.uint8), fun="sum", encoding="numpy")
    assert r.shape == (1, 131, 361)
    assert np.array_equal(r[0], np.load(GOLDEN / "standard_output_sum.npy"))
    # test_many.py:116-123
    r2 = rz.rusterize(geoms, res=(1, 1), burn=99, encoding="numpy").squeeze()
    assert np.nanmax(r2) == 99
    assert np.nanmin(r2[r2 > 0]) == 99
    r3 = rz.rusterize(geoms, res=(1, 1), burn=1, background=-1, encoding="numpy").squeeze()
    assert r3[0, 0] == -1


def test_dedup_in_big_buckets():
    # > 256 and > 4096 spans of deduplicating line parts in one row tile
    b = G.TableBuilder()
    rng = np.random.default_rng(33)
    segs = []
    for i in range(5000):
        x = float(rng.uniform(0, 900))
        segs.append([(x, 0.5), (x + float(rng.uniform(0.5, 40)), 0.5)])
    G.add_multilinestring(b, segs)           # one part, thousands of overlapping runs
    for i in range(400):
        x = float(rng.uniform(0, 900))
        G.add_linestring(b, [(x, 0.2), (x + 30, 0.9), (x + 5, 0.3)])
    t = b.build()
    grid = dict(nrows=1, ncols=1000, xmin=0.0, xmax=1000.0, ymin=0.0, ymax=1.5, xres=1.0, yres=1.5)
    for fn in ("sum", "count"):
        check(t, grid, fn=fn, values=np.arange(1.0, t.n_geoms + 1), background=0.0)
