"""SparseArray::build_array (rust/src/encoding/arrays.rs:103-141): a COO
triplet stream replayed onto a background raster with the pixel function,
each band's triplets in stream order.

On the CPU the oracle's replay is pinned to the oracle's dense burn: the
sparse stream of a burn, replayed, is that burn's raster, for every pixel
function.  On the GPU ``rz_sparse_build`` is compared bit for bit with the
oracle's replay -- on the streams of real burns, and on synthetic streams
that write each pixel many times in random order with values equal to the
background, NaN and signed zeros, which is where the order of one pixel's
writes decides the result (a write that leaves a pixel at the background
resets it for the next write).  A stream longer than one replay chunk
(2^28 triplets) checks that chunks fold onto the raster in order."""

import zlib

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth
from rusterize_gb300.engine import RasterInfo, rasterize_table_sparse, sparse_build

import oracle
from _util import diff_report, same_bits

FNS = ["sum", "first", "last", "min", "max", "count", "any"]
DTYPES = ["uint8", "int16", "uint32", "int64", "float32", "float64"]


def _mixed(seed, side, n=120):
    rng = np.random.default_rng(seed)
    polys = synth.star_polygons(rng, n, (3, 30), rng.uniform(1.0, 25.0, n), rng.uniform(-20, side + 20, n),
                                rng.uniform(-20, side + 20, n), n_holes=rng.integers(0, 3, n))
    lines = synth.random_walk_lines(rng, n // 2, (2, 30), (0.3, 12.0), (-10, -10, side + 10, side + 10))
    pts = synth.random_points(rng, n // 2, (0, 0, side, side))
    return G.GeometryTable.concat([polys, lines, pts]), rng


def _values(rng, n, dtype, bg):
    """Values with many collisions with the background, plus NaN and -0.0
    for floating point outputs."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        v = rng.integers(-3, 4, n).astype(dt)
        v[rng.random(n) < 0.05] = np.nan
        v[rng.random(n) < 0.05] = -0.0
        if not np.isnan(bg):
            v[rng.random(n) < 0.1] = bg
        return v
    info = np.iinfo(dt)
    v = rng.integers(max(info.min, -3), min(info.max, 250) + 1, n).astype(dt)
    v[rng.random(n) < 0.1] = np.array(bg).astype(dt)
    return v


def _stream(rng, n_bands, nrows, ncols, per_band, dtype, bg):
    counts = np.array(per_band, dtype=np.uint64)
    n = int(counts.sum())
    rows = rng.integers(0, nrows, n).astype(np.uint64)
    cols = rng.integers(0, ncols, n).astype(np.uint64)
    return counts, rows, cols, _values(rng, n, dtype, bg)


# ---------------------------------------------------------------- CPU ------
@pytest.mark.parametrize("fn", FNS)
def test_oracle_replay_of_a_sparse_burn_is_the_dense_burn(fn):
    t, rng = _mixed(3, 80)
    v = rng.integers(1, 9, t.n_geoms).astype(np.float32)
    bands = (np.arange(t.n_geoms) % 3).astype(np.uint32)
    g = dict(nrows=80, ncols=80, xmin=0.0, xmax=80.0, ymin=0.0, ymax=80.0, xres=1.0, yres=1.0)
    for bg in (0.0, np.nan):
        bc, rows, cols, vals = oracle.rasterize_sparse(t, g["nrows"], g["ncols"], g["xmin"], g["xmax"], g["ymin"],
                                                       g["ymax"], g["xres"], g["yres"], values=v, fn=fn,
                                                       dtype="float32", bands=bands, n_bands=3)
        replay = oracle.sparse_build(bc, rows, cols, vals, 80, 80, fn=fn, background=bg)
        dense = oracle.rasterize(t, g["nrows"], g["ncols"], g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["xres"],
                                 g["yres"], values=v, fn=fn, background=bg, dtype="float32", bands=bands,
                                 n_bands=3)
        assert same_bits(replay, dense), diff_report(replay, dense)


def test_oracle_replay_applies_writes_in_stream_order():
    # one pixel: sum with background 0 -- 2 + (-2) leaves 0 (the background), so 5 starts over
    out = oracle.sparse_build([3], [0, 0, 0], [0, 0, 0], np.array([2.0, -2.0, 5.0]), 1, 1, fn="sum", background=0.0)
    assert out.tolist() == [[[5.0]]]
    out = oracle.sparse_build([3], [0, 0, 0], [0, 0, 0], np.array([5.0, 2.0, -2.0]), 1, 1, fn="sum", background=0.0)
    assert out.tolist() == [[[5.0]]]
    out = oracle.sparse_build([2, 1], [0, 0, 0], [1, 1, 1], np.array([7, 9, 4], np.int32), 1, 2, fn="first",
                              background=0)
    assert out.tolist() == [[[0, 7]], [[0, 4]]]
    with pytest.raises(ValueError, match="outside"):
        oracle.sparse_build([1], [1], [0], np.array([1.0]), 1, 1, fn="last", background=0.0)


# ---------------------------------------------------------------- GPU ------
@pytest.mark.gpu
@pytest.mark.parametrize("fn", FNS)
def test_replay_of_burn_streams_matches_the_oracle(fn):
    t, rng = _mixed(5, 96)
    info = RasterInfo(96, 96, 0.0, 96.0, 0.0, 96.0, 1.0, 1.0)
    bands = (np.arange(t.n_geoms) % 4).astype(np.uint32)
    for dtype in ("float64", "int32"):
        v = rng.integers(-4, 9, t.n_geoms).astype(dtype)
        bc, rows, cols, vals = rasterize_table_sparse(t, info, values=v, fn=fn, dtype=dtype, bands=bands,
                                                      n_bands=4)
        for bg in (0, 3) if dtype == "int32" else (0.0, np.nan):
            got = sparse_build(bc, rows, cols, vals, 96, 96, fn=fn, background=bg)
            ref = oracle.sparse_build(bc, rows, cols, vals, 96, 96, fn=fn, background=bg)
            assert same_bits(got, ref), f"{dtype} bg={bg}: " + diff_report(got, ref)
            dense = rz.rasterize_table(t, info, values=v, fn=fn, background=bg, dtype=dtype, bands=bands,
                                       n_bands=4)
            assert same_bits(got, dense)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("fn", FNS)
def test_replay_of_random_streams_matches_the_oracle(fn, dtype):
    """Each pixel written ~40 times in random order, values colliding with
    the background; several bands, one of them empty."""
    rng = np.random.default_rng(zlib.crc32(f"{fn}/{dtype}".encode()))
    bgs = (0, 5) if np.dtype(dtype).kind != "f" else (0.0, np.nan, 5.0)
    for bg in bgs:
        counts, rows, cols, vals = _stream(rng, 3, 17, 23, [6000, 0, 9000], dtype, bg)
        got = sparse_build(counts, rows, cols, vals, 17, 23, fn=fn, background=bg)
        ref = oracle.sparse_build(counts, rows, cols, vals, 17, 23, fn=fn, background=bg)
        assert same_bits(got, ref), f"bg={bg}: " + diff_report(got, ref)


@pytest.mark.gpu
def test_replay_edge_cases():
    # no triplets: the background raster
    got = sparse_build([0, 0], np.zeros(0, np.uint64), np.zeros(0, np.uint64), np.zeros(0, np.float32), 3, 4,
                       fn="sum", background=np.nan)
    assert got.shape == (2, 3, 4) and np.isnan(got).all()
    # an empty raster with no triplets
    assert sparse_build([0], [], [], np.zeros(0, np.uint8), 0, 5, fn="any", background=0).shape == (1, 0, 5)
    # a triplet outside the raster is refused (the reference's indexing panics)
    for r, c in ((3, 0), (0, 4), (2**63, 0)):
        with pytest.raises(ValueError, match="outside the raster"):
            sparse_build([2], [0, r], [0, c], np.array([1.0, 2.0]), 3, 4, fn="last", background=0.0)
    # the context is still usable afterwards
    got = sparse_build([2], [0, 2], [0, 3], np.array([1.0, 2.0]), 3, 4, fn="last", background=0.0)
    assert got[0, 0, 0] == 1.0 and got[0, 2, 3] == 2.0 and got.sum() == 3.0
    with pytest.raises(ValueError, match="disagree"):
        sparse_build([3], [0, 1], [0, 1], np.array([1.0, 2.0]), 3, 4, fn="last", background=0.0)


@pytest.mark.gpu
def test_replay_across_chunks_keeps_stream_order():
    """2^28 + 4,321 triplets over a 64 x 64 raster (about 65,000 writes per
    pixel, the chunk boundary inside every pixel's sequence): `count` equals
    the histogram of the pixels and `last` the value of each pixel's last
    triplet in the stream."""
    n = (1 << 28) + 4321
    rng = np.random.default_rng(17)
    key = rng.integers(0, 64 * 64, n, dtype=np.int64)
    rows = (key // 64).astype(np.uint64)
    cols = (key % 64).astype(np.uint64)
    vals = rng.integers(1, 1 << 20, n).astype(np.float32)
    cnt = sparse_build([n], rows, cols, np.ones(n, np.uint32), 64, 64, fn="count", background=0)
    assert np.array_equal(cnt.reshape(-1), np.bincount(key, minlength=64 * 64).astype(np.uint32))
    last = sparse_build([n], rows, cols, vals, 64, 64, fn="last", background=0.0)
    last_ix = np.full(64 * 64, -1, np.int64)
    np.maximum.at(last_ix, key, np.arange(n, dtype=np.int64))
    assert (last_ix >= 0).all()
    assert same_bits(last.reshape(-1), vals[last_ix])
