"""Burning a window of the raster's rows (rz_rasterize_rows), and rasters
with more (band, row, tile) buckets than one pass holds.

* A window [r0, r1) must equal rows r0..r1 of the whole burn bit for bit:
  polygon scanlines, Bresenham and AllTouched walks, the end pixel of a
  line's last kept segment and points are all decided on the whole raster's
  grid and only clipped to the window.
* A raster of more than 2^28 - 1 buckets is burned in passes of one band and
  a run of rows each; the result must equal the oracle's.  A one-column
  raster reaches that count with little memory (one bucket per row).
"""

from __future__ import annotations

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth

from _util import diff_report, gpu_burn, oracle_burn, same_bits

pytestmark = pytest.mark.gpu


def _mixed_small():
    a, b = synth.mixed(seed=77, scale=0.0005)
    return a, b


@pytest.mark.parametrize("fn,dtype,bg", [("sum", "float64", np.nan), ("count", "uint32", 0), ("last", "float32", -1.0),
                                         ("max", "int32", 0)])
@pytest.mark.parametrize("all_touched", [False, True])
def test_row_windows_equal_slices_of_the_whole_burn(fn, dtype, bg, all_touched):
    a, b = _mixed_small()
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    vals = np.arange(a.table.n_geoms) % 13 + 1
    whole = gpu_burn(a.table, info, fn=fn, values=vals, background=bg, dtype=dtype, all_touched=all_touched)
    ref = oracle_burn(a.table, info, fn=fn, values=vals, background=bg, dtype=dtype, all_touched=all_touched)
    assert same_bits(whole, ref), diff_report(whole, ref)
    n = info.nrows
    for r0, r1 in [(0, n), (0, 1), (n - 1, n), (3, 700), (511, 513), (n // 3, 2 * n // 3), (5, 5)]:
        got = rz.rasterize_table(a.table, info, values=vals.astype(dtype), fn=fn, background=bg, dtype=dtype,
                                 all_touched=all_touched, rows=(r0, r1))
        assert got.shape == (1, r1 - r0, info.ncols)
        assert same_bits(got, whole[:, r0:r1]), f"rows {r0}:{r1}: " + diff_report(got, whole[:, r0:r1])


def test_row_windows_with_bands_and_non_square_pixels():
    a, _ = _mixed_small()
    info = rz.raster_info(a.table, res=(1.3, 0.7), extent=a.extent)
    whole = gpu_burn(a.table, info, fn="sum", background=0, dtype="uint16", bands=a.bands, n_bands=a.n_bands)
    for r0, r1 in [(0, 17), (100, 900), (info.nrows - 300, info.nrows)]:
        got = rz.rasterize_table(a.table, info, fn="sum", background=0, dtype="uint16", bands=a.bands,
                                 n_bands=a.n_bands, rows=(r0, r1))
        assert same_bits(got, whole[:, r0:r1])


def test_row_window_outside_the_raster_is_refused():
    a, _ = _mixed_small()
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    with pytest.raises(ValueError):
        rz.rasterize_table(a.table, info, fn="count", background=0, dtype="uint8", rows=(10, info.nrows + 1))


def test_more_than_2_28_buckets_in_passes_against_oracle():
    # 16 bands x (2^24 + 100) rows x 1 column: 268,437,056 buckets > 2^28 - 1
    nrows = (1 << 24) + 100
    rng = np.random.default_rng(5)
    b = G.TableBuilder()
    bands = []
    for i in range(400):
        y = float(rng.uniform(0, nrows))
        kind = i % 3
        if kind == 0:
            G.add_polygon(b, [(-0.5, y), (1.5, y + 3.5), (0.2, y + 9.0), (-0.5, y)])
        elif kind == 1:
            G.add_linestring(b, [(0.3, y), (0.6, y + 40.0), (0.4, y + 45.0)])
        else:
            G.add_point(b, 0.5, y)
        bands.append(int(rng.integers(0, 16)))
    # a few geometries straddling the pass boundary of band 0
    for y in ((1 << 24) + 50.0, float((1 << 28) - 1 - (1 << 24) * 15) - 2.0):
        G.add_polygon(b, [(-1.0, y - 5.0), (2.0, y - 5.0), (2.0, y + 5.0), (-1.0, y + 5.0), (-1.0, y - 5.0)])
        bands.append(0)
    t = b.build()
    bands = np.array(bands, dtype=np.uint32)
    info = rz.RasterInfo(nrows, 1, 0.0, 1.0, 0.0, float(nrows), 1.0, 1.0)
    vals = (np.arange(t.n_geoms) % 200 + 1).astype(np.uint8)
    st: dict = {}
    got = gpu_burn(t, info, fn="sum", values=vals, background=0, dtype="uint8", bands=bands, n_bands=16, stats=st)
    assert st["buckets"] == 16 * nrows
    ref = oracle_burn(t, info, fn="sum", values=vals, background=0, dtype="uint8", bands=bands, n_bands=16)
    assert same_bits(got, ref), diff_report(got, ref)
    assert int(ref.astype(np.uint64).sum()) > 0


def test_polygons_wider_than_one_bitmap_against_oracle():
    """Parts wider than the 8,192-word (262,144-pixel) bitmap burn in column
    windows: crossings left of a window flip its rows' parity, the largest
    crossing of an odd row is dropped wherever it lies.  A 400,000-column
    raster, 300 rows: long thin polygons, a huge star polygon (most of whose
    edges miss the rows) with a hole, and small ones on top, checked with
    `sum` (order) and `count` against the oracle."""
    rng = np.random.default_rng(21)
    ncols, nrows = 400_000, 300
    b = G.TableBuilder()
    # a band across the whole width with a notch, and a sliver
    G.add_polygon(b, [(-10.0, 20.5), (400_010.0, 35.2), (399_000.0, 120.0), (200_000.0, 90.0), (-5.0, 140.0)])
    G.add_polygon(b, [(1000.5, 200.0), (350_000.25, 205.0), (1000.5, 210.0)])
    # a star polygon of radius ~190k centred on the raster, with a hole
    n = 300
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    rad = 190_000.0 * rng.uniform(0.4, 1.0, n)
    ext = np.stack([200_000.0 + rad * np.cos(ang), 150.0 + rad * np.sin(ang) * 0.001], axis=1)
    hole = np.array([[150_000.0, 140.0], [250_000.0, 145.0], [240_000.0, 160.0], [160_000.0, 158.0]])
    G.add_polygon(b, ext, [hole])
    for _ in range(200):  # small polygons everywhere
        cx, cy = rng.uniform(0, ncols), rng.uniform(0, nrows)
        k = int(rng.integers(5, 30))
        a = np.sort(rng.uniform(0, 2 * np.pi, k))
        r = rng.uniform(2, 40, k)
        G.add_polygon(b, np.stack([cx + r * np.cos(a), cy + r * np.sin(a)], axis=1))
    t = b.build()
    info = rz.RasterInfo(nrows, ncols, 0.0, float(ncols), 0.0, float(nrows), 1.0, 1.0)
    vals = (np.arange(t.n_geoms) % 17 + 1).astype(np.float64)
    for fn, dt, bg in (("sum", "float64", np.nan), ("count", "uint32", 0)):
        v = vals if fn == "sum" else None
        got = gpu_burn(t, info, fn=fn, values=v, background=bg, dtype=dt)
        ref = oracle_burn(t, info, fn=fn, values=v, background=bg, dtype=dt)
        assert same_bits(got, ref), f"{fn}: " + diff_report(got, ref)
    # the windows also hold with a row window and all_touched
    got = rz.rasterize_table(t, info, fn="count", background=0, dtype="uint32", rows=(100, 180))
    assert same_bits(got, ref[:, 100:180])
    got = gpu_burn(t, info, fn="max", values=vals, background=0.0, dtype="float64", all_touched=True)
    ref = oracle_burn(t, info, fn="max", values=vals, background=0.0, dtype="float64", all_touched=True)
    assert same_bits(got, ref), "all_touched: " + diff_report(got, ref)
