"""CPU oracle of rusterize's burn path -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper of ``oracle/_build/librz_oracle.so`` (built from
``oracle/rz_oracle.cpp`` by ``oracle/build.py``), a restatement of the Rust
reference (ttrotto/rusterize, rust/src/) pinned against the reference's
golden rasters and known-answer tests.  Only tests/, the smoke check and
bench.py's CPU-baseline legs use it; the engine never does.

Inputs are duck-typed geometry tables: any object with ``part_offsets``,
``part_kind``, ``ring_offsets``, ``vertex_offsets``, ``ring_flags`` and
``xy`` numpy arrays (the engine's flat "parts" layout).
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_uint8, c_uint32, c_uint64, c_void_p

import numpy as np

from .build import build

DTYPES = {
    "uint8": 0, "uint16": 1, "uint32": 2, "uint64": 3,
    "int8": 4, "int16": 5, "int32": 6, "int64": 7,
    "float32": 8, "float64": 9,
}
PIXEL_FNS = {"sum": 0, "first": 1, "last": 2, "min": 3, "max": 4, "count": 5, "any": 6}
RI_ERRORS = {
    1: (ValueError, "Unspecified extent (all zeros)."),
    2: (RuntimeError, "Cannot infer bounding box from geometry."),
    3: (ValueError, "Must set at least one of `shape` or `resolution`"),
    4: (ValueError, "Shape and resolution are mutually exclusive; provide only one"),
    5: (ValueError, "Shape values must be > 0."),
    6: (ValueError, "Resolution values must be > 0."),
}

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        lib.rzo_rasterize.restype = c_int
        lib.rzo_rasterize.argtypes = [c_uint64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                      c_void_p, c_uint32, c_void_p, c_uint64, c_uint64, c_int, c_void_p, c_int,
                                      c_void_p, POINTER(c_uint64), POINTER(c_uint64)]
        lib.rzo_raster_info.restype = c_int
        lib.rzo_raster_info.argtypes = [c_uint64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        lib.rzo_rasterize_sparse.restype = c_int
        lib.rzo_rasterize_sparse.argtypes = [c_uint64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                             c_int, c_void_p, c_uint32, c_void_p, c_uint64, c_uint64, c_int, c_int,
                                             POINTER(c_uint64), POINTER(c_void_p), POINTER(c_void_p),
                                             POINTER(c_void_p), c_void_p]
        lib.rzo_sparse_build.restype = c_int
        lib.rzo_sparse_build.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_int, c_uint64, c_uint64,
                                         c_int, c_void_p, c_void_p]
        lib.rzo_free.restype = None
        lib.rzo_free.argtypes = [c_void_p]
        _lib = lib
    return _lib


def _arrays(t):
    return (np.ascontiguousarray(t.part_offsets, np.uint64), np.ascontiguousarray(t.part_kind, np.uint8),
            np.ascontiguousarray(t.ring_offsets, np.uint64), np.ascontiguousarray(t.vertex_offsets, np.uint64),
            np.ascontiguousarray(t.ring_flags, np.uint8), np.ascontiguousarray(t.xy, np.float64))


def raster_info(table, shape=None, res=None, extent=None, tap=False):
    """RasterInfoBuilder restatement; returns (nrows, ncols, xmin, xmax, ymin, ymax, xres, yres)."""
    lib = load()
    po, pk, ro, vo, rf, xy = _arrays(table)
    flags = (1 if shape is not None else 0) | (2 if res is not None else 0) | (4 if extent is not None else 0) | (
        8 if tap else 0)
    c_shape = np.array(shape if shape is not None else (0, 0), np.uint64)
    c_res = np.array(res if res is not None else (0, 0), np.float64)
    c_ext = np.array(extent if extent is not None else (0, 0, 0, 0), np.float64)
    info = np.zeros(6, np.float64)
    oshape = np.zeros(2, np.uint64)
    st = lib.rzo_raster_info(len(po) - 1, po.ctypes.data, pk.ctypes.data, ro.ctypes.data, vo.ctypes.data,
                             rf.ctypes.data, xy.ctypes.data, flags, c_shape.ctypes.data, c_res.ctypes.data,
                             c_ext.ctypes.data, info.ctypes.data, oshape.ctypes.data)
    if st:
        exc, msg = RI_ERRORS[st]
        raise exc(msg)
    return (int(oshape[0]), int(oshape[1]), *map(float, info))


def rasterize(table, nrows, ncols, xmin, xmax, ymin, ymax, xres, yres, *, values=None, fn="last", background=0,
              dtype="float64", bands=None, n_bands=None, all_touched=False, counters=None):
    """Burn with the CPU restatement.  Returns (bands, nrows, ncols) of dtype.

    values: None (T::one()), a scalar, or a per-geometry array (cast to dtype).
    """
    lib = load()
    po, pk, ro, vo, rf, xy = _arrays(table)
    dt = np.dtype(dtype)
    G = len(po) - 1
    if values is None:
        vals = None
    elif np.isscalar(values) or (isinstance(values, np.ndarray) and values.ndim == 0):
        vals = np.full(G, values, dtype=dt)
    else:
        vals = np.ascontiguousarray(values, dtype=dt)
    if bands is not None:
        bands = np.ascontiguousarray(bands, np.uint32)
        nb = int(n_bands if n_bands is not None else (bands.max() + 1 if len(bands) else 1))
    else:
        nb = 1
    out = np.empty((nb, nrows, ncols), dtype=dt)
    bg = np.array([background], dtype=dt)
    raster = np.array([xmin, xmax, ymin, ymax, xres, yres], np.float64)
    nw, ne = c_uint64(0), c_uint64(0)
    st = lib.rzo_rasterize(G, po.ctypes.data, pk.ctypes.data, ro.ctypes.data, vo.ctypes.data, xy.ctypes.data,
                           None if vals is None else vals.ctypes.data, DTYPES[dt.name],
                           None if bands is None else bands.ctypes.data, nb, raster.ctypes.data, nrows, ncols,
                           PIXEL_FNS[fn], bg.ctypes.data, int(bool(all_touched)), out.ctypes.data,
                           ctypes.byref(nw), ctypes.byref(ne))
    if st:
        raise ValueError(f"oracle failed with status {st}")
    if counters is not None:
        counters["pixel_writes"] = nw.value
        counters["edges"] = ne.value
    return out


def rasterize_sparse(table, nrows, ncols, xmin, xmax, ymin, ymax, xres, yres, *, values=None, fn="last",
                     dtype="float64", bands=None, n_bands=None, all_touched=False):
    """Sparse burn with the CPU restatement: (band_counts, rows, cols, values)
    in the reference's write order (SparseArrayWriter, writers.rs:86-131)."""
    lib = load()
    po, pk, ro, vo, rf, xy = _arrays(table)
    dt = np.dtype(dtype)
    G = len(po) - 1
    if values is None:
        vals = None
    elif np.isscalar(values) or (isinstance(values, np.ndarray) and values.ndim == 0):
        vals = np.full(G, values, dtype=dt)
    else:
        vals = np.ascontiguousarray(values, dtype=dt)
    if bands is not None:
        bands = np.ascontiguousarray(bands, np.uint32)
        nb = int(n_bands if n_bands is not None else (bands.max() + 1 if len(bands) else 1))
    else:
        nb = 1
    raster = np.array([xmin, xmax, ymin, ymax, xres, yres], np.float64)
    count = c_uint64(0)
    rows_p, cols_p, vals_p = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    band_counts = np.zeros(nb, np.uint64)
    st = lib.rzo_rasterize_sparse(G, po.ctypes.data, pk.ctypes.data, ro.ctypes.data, vo.ctypes.data, xy.ctypes.data,
                                  None if vals is None else vals.ctypes.data, DTYPES[dt.name],
                                  None if bands is None else bands.ctypes.data, nb, raster.ctypes.data, nrows, ncols,
                                  PIXEL_FNS[fn], int(bool(all_touched)), ctypes.byref(count), ctypes.byref(rows_p),
                                  ctypes.byref(cols_p), ctypes.byref(vals_p), band_counts.ctypes.data)
    if st:
        raise ValueError(f"oracle failed with status {st}")
    n = count.value
    try:
        rows = np.ctypeslib.as_array(ctypes.cast(rows_p, ctypes.POINTER(ctypes.c_uint64)), (max(n, 1),))[:n].copy()
        cols = np.ctypeslib.as_array(ctypes.cast(cols_p, ctypes.POINTER(ctypes.c_uint64)), (max(n, 1),))[:n].copy()
        if n:
            raw = np.ctypeslib.as_array(ctypes.cast(vals_p, ctypes.POINTER(ctypes.c_uint8)), shape=(n * dt.itemsize,))
            out_vals = raw.view(dt).copy()
        else:
            out_vals = np.empty(0, dtype=dt)
    finally:
        for p_ in (rows_p, cols_p, vals_p):
            lib.rzo_free(p_)
    return band_counts, rows, cols, out_vals


def sparse_build(band_counts, rows, cols, values, nrows, ncols, *, fn="last", background=0):
    """SparseArray::build_array with the CPU restatement: the triplet stream
    (band_counts[b] triplets for band b, bands in order) replayed onto a
    (bands, nrows, ncols) background raster of the values' dtype."""
    lib = load()
    counts = np.ascontiguousarray(band_counts, np.uint64)
    rows = np.ascontiguousarray(rows, np.uint64)
    cols = np.ascontiguousarray(cols, np.uint64)
    vals = np.ascontiguousarray(values)
    dt = vals.dtype
    out = np.empty((len(counts), int(nrows), int(ncols)), dtype=dt)
    bg = np.array([background], dtype=dt)
    st = lib.rzo_sparse_build(counts.ctypes.data, len(counts), rows.ctypes.data, cols.ctypes.data, vals.ctypes.data,
                              DTYPES[dt.name], nrows, ncols, PIXEL_FNS[fn], bg.ctypes.data, out.ctypes.data)
    if st == -3:
        raise ValueError("triplet outside the raster")
    if st:
        raise ValueError(f"oracle failed with status {st}")
    return out
