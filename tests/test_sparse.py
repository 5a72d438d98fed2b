"""The sparse (COO) encoding on the GPU against the oracle's SparseArrayWriter
stream (rust/src/encoding/writers.rs:86-131, SparseArray in
rust/src/encoding/arrays.rs:62-209), through the C ABI.

The GPU stream holds the same (band, row, col, value) triplets as the
reference's, grouped by band in band order, and every pixel sees its writes
in the same order; only the order of one geometry's own triplets differs
(row by row on the GPU).  So the two streams are compared after a stable
sort by (band, row, col): equal, bit for bit, including the per-band counts.
On larger jobs the checks are size-independent: the number of triplets of a
``count`` burn equals the sum of the dense ``count`` raster, an integer
``sum`` replayed from the triplets equals the dense ``sum`` raster, and
``to_numpy`` equals the dense encoding."""

import zlib

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth
from rusterize_gb300.engine import RasterInfo, rasterize_table, rasterize_table_sparse

import oracle
from _util import diff_report, grid_of, same_bits

pytestmark = pytest.mark.gpu

FNS = ["sum", "first", "last", "min", "max", "count", "any"]


def _canon(band_counts, rows, cols, vals):
    band = np.repeat(np.arange(len(band_counts), dtype=np.uint64), band_counts.astype(np.int64))
    order = np.lexsort((cols, rows, band))  # stable: ties keep stream order
    return band[order], rows[order], cols[order], vals[order]


def check(table, grid, **kw):
    g = grid_of(grid)
    info = RasterInfo(**g)
    got = rasterize_table_sparse(table, info, **kw)
    ref = oracle.rasterize_sparse(table, g["nrows"], g["ncols"], g["xmin"], g["xmax"], g["ymin"], g["ymax"],
                                  g["xres"], g["yres"], **kw)
    assert np.array_equal(got[0], ref[0]), f"band counts {got[0]} != {ref[0]}"
    a, b = _canon(*got), _canon(*ref)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), \
        "triplet coordinates differ"
    assert same_bits(a[3], b[3]), diff_report(a[3], b[3])
    return got


def _grid(n, m=None, res=(1.0, 1.0)):
    m = n if m is None else m
    return dict(nrows=n, ncols=m, xmin=0.0, xmax=m * res[0], ymin=0.0, ymax=n * res[1], xres=res[0], yres=res[1])


def _mixed(seed, side, n=150):
    rng = np.random.default_rng(seed)
    polys = synth.star_polygons(rng, n, (3, 30), rng.uniform(1.0, 25.0, n), rng.uniform(-20, side + 20, n),
                                rng.uniform(-20, side + 20, n), n_holes=rng.integers(0, 3, n))
    lines = synth.random_walk_lines(rng, n // 2, (2, 30), (0.3, 12.0), (-10, -10, side + 10, side + 10))
    pts = synth.random_points(rng, n // 2, (0, 0, side, side))
    return G.GeometryTable.concat([polys, lines, pts]), rng


@pytest.mark.parametrize("touched", [False, True])
@pytest.mark.parametrize("fn", FNS)
def test_every_function_matches_the_oracle_stream(fn, touched):
    t, rng = _mixed(zlib.crc32(fn.encode()) + touched, 130)
    v = rng.integers(1, 6, t.n_geoms).astype(np.float64)
    check(t, _grid(130), fn=fn, values=v, dtype="float64", all_touched=touched)


@pytest.mark.parametrize("dtype", ["uint8", "int16", "uint32", "int64", "float32"])
def test_dtypes_bands_and_non_square_pixels(dtype):
    t, rng = _mixed(zlib.crc32(dtype.encode()), 200, n=200)
    n_bands = 4
    bands = rng.integers(0, n_bands, t.n_geoms).astype(np.uint32)
    bands[bands == 2] = 3  # band 3 of 4 stays empty
    v = rng.integers(0, 100, t.n_geoms).astype(dtype)
    check(t, _grid(170, 230, res=(200 / 230, 200 / 170)), fn="sum", values=v, dtype=dtype, bands=bands,
          n_bands=n_bands)
    check(t, _grid(170, 230, res=(200 / 230, 200 / 170)), fn="last", values=v, dtype=dtype, bands=bands,
          n_bands=n_bands, all_touched=True)


def test_scalar_and_default_values():
    t, _ = _mixed(5, 90)
    check(t, _grid(90), fn="sum", values=2.5, dtype="float32")
    check(t, _grid(90), fn="last", values=None, dtype="uint16")


def test_nothing_burned():
    b = G.TableBuilder()
    G.add_polygon(b, np.array([[500.0, 500.0], [510.0, 500.0], [510.0, 510.0], [500.0, 500.0]]))
    G.add_linestring(b, [(-50.0, -50.0), (-40.0, -45.0)])
    G.add_point(b, 1e6, 1e6)
    bc, rows, cols, vals = check(b.build(), _grid(64), fn="sum", values=np.array([1.0, 2.0, 3.0]))
    assert bc.tolist() == [0] and len(rows) == len(cols) == len(vals) == 0


def test_one_geometry_many_parts_overlapping_lines():
    # self-crossing and repeated line parts: the deduplicated functions
    # (sum, count) write a pixel once per geometry, the others once per visit
    b = G.TableBuilder()
    parts = [[(0.5, 0.5), (30.5, 20.5), (0.5, 20.5), (30.5, 0.5)], [(0.5, 0.5), (30.5, 20.5)],
             [(3.0, 29.0), (3.0, 1.0), (28.0, 1.0)]]
    G.add_multilinestring(b, parts)
    t = b.build()
    for fn in ("sum", "count", "last", "min"):
        for touched in (False, True):
            check(t, _grid(32), fn=fn, values=np.array([4.0]), all_touched=touched)


def test_sparse_array_object_mirrors_the_reference():
    t, rng = _mixed(11, 100)
    v = rng.integers(1, 9, t.n_geoms).astype(np.float64)
    by = [("a", "b", "c")[i % 3] for i in range(t.n_geoms)]
    # through the native entry point with a dict frame (columns by name)
    sp = rz._rusterize(t, {"resolution": (1.0, 1.0), "extent": (0.0, 0.0, 100.0, 100.0)}, "sum",
                       {"v": list(v), "by": by}, "v", "by", None, 0.0, False, "sparse", "float64")
    assert isinstance(sp, rz.SparseArray)
    assert sp.shape() == (3, 100, 100)
    assert sp.band_names() == ["a", "b", "c"]
    assert repr(sp).startswith("SparseArray:\n- Shape: (3, 100, 100)\n- Extent: (0.0, 0.0, 100.0, 100.0)\n")
    assert repr(sp).endswith("- EPSG: None\n- Estimated size: 240.00 KB")
    dense = rz._rusterize(t, {"resolution": (1.0, 1.0), "extent": (0.0, 0.0, 100.0, 100.0)}, "sum",
                          {"v": list(v), "by": by}, "v", "by", None, 0.0, False, "numpy", "float64")
    assert same_bits(sp.to_numpy(), dense)
    trip = sp.triplets()
    assert list(trip) == ["band", "row", "col", "values"]
    assert len(trip["band"]) == len(trip["row"]) and trip["band"].min() == 1 and trip["band"].max() == 3


def test_large_size_properties():
    """Size-independent checks on larger jobs: the 16-band mixed workload
    (polygons, lines, points) at 2% of its area and the large polygon
    workload at 5%: triplets per band vs the dense `count` raster, integer
    sums replayed from the triplets vs the dense `sum` raster."""
    a, _ = synth.mixed(1003, scale=0.02)
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    dense_count = rasterize_table(a.table, info, fn="count", dtype="uint16", bands=a.bands, n_bands=a.n_bands)
    bc, rows, cols, vals = rasterize_table_sparse(a.table, info, fn="count", dtype="uint16", bands=a.bands,
                                                  n_bands=a.n_bands)
    assert bc.tolist() == dense_count.reshape(a.n_bands, -1).sum(axis=1, dtype=np.uint64).tolist()
    assert (vals == 1).all()
    w = synth.large_fill(1002, scale=0.05)
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    iv = (np.arange(w.table.n_geoms) % 97 + 1).astype(np.int64)
    dense = rasterize_table(w.table, info, fn="sum", values=iv, dtype="int64", background=0)
    bc, rows, cols, vals = rasterize_table_sparse(w.table, info, fn="sum", values=iv, dtype="int64")
    assert int(bc[0]) == len(rows) and rows.max() < info.nrows and cols.max() < info.ncols
    # integer sums far below 2**53: the float64 bincount is exact
    replay = np.bincount((rows * np.uint64(info.ncols) + cols).astype(np.int64), weights=vals.astype(np.float64),
                         minlength=info.nrows * info.ncols)
    assert np.array_equal(replay.astype(np.int64).reshape(dense.shape[1:]), dense[0])
