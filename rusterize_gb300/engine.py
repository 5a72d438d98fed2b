"""Thin typed wrappers over the engine's C ABI: raster-grid building and the
dense burn call.  Everything computes on the GPU; nothing here falls back to
the CPU."""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _lib
from .geometry import GeometryTable


@dataclass
class RasterInfo:
    """rust/src/geo/raster.rs:8-20.  Row 0 is the ymax edge."""

    nrows: int
    ncols: int
    xmin: float
    xmax: float
    ymin: float
    ymax: float
    xres: float
    yres: float
    epsg: int | None = None

    def c_struct(self) -> _lib.RzRasterInfo:
        r = _lib.RzRasterInfo()
        r.nrows, r.ncols = self.nrows, self.ncols
        r.xmin, r.xmax, r.ymin, r.ymax = self.xmin, self.xmax, self.ymin, self.ymax
        r.xres, r.yres = self.xres, self.yres
        r.epsg = -1 if self.epsg is None else int(self.epsg)
        return r

    @property
    def shape(self) -> tuple[int, int]:
        return (self.nrows, self.ncols)


def raster_info(table: GeometryTable | None, shape=None, res=None, extent=None, tap: bool = False,
                epsg: int | None = None) -> RasterInfo:
    """RawRasterInfo::build (python/src/geo/raster.rs:17-41).  Errors are the
    reference's RusterizeError strings, raised as ValueError/RuntimeError."""
    lib = _lib.load()
    flags = 0
    c_shape = (ctypes.c_uint64 * 2)(0, 0)
    c_res = (ctypes.c_double * 2)(0.0, 0.0)
    c_ext = (ctypes.c_double * 4)(0.0, 0.0, 0.0, 0.0)
    if shape is not None:
        flags |= _lib.RI_SHAPE
        c_shape[0], c_shape[1] = int(shape[0]), int(shape[1])
    if res is not None:
        flags |= _lib.RI_RES
        c_res[0], c_res[1] = float(res[0]), float(res[1])
    if extent is not None:
        flags |= _lib.RI_EXTENT
        for i in range(4):
            c_ext[i] = float(extent[i])
    if tap:
        flags |= _lib.RI_TAP
    g = table.c_view() if table is not None else None
    out = _lib.RzRasterInfo()
    e = _lib.errbuf()
    st = lib.rz_raster_info_build(ctypes.byref(g) if g is not None else None, flags, c_shape, c_res, c_ext,
                                  -1 if epsg is None else int(epsg), ctypes.byref(out), e, len(e))
    _lib.raise_for(st, e.value)
    return RasterInfo(out.nrows, out.ncols, out.xmin, out.xmax, out.ymin, out.ymax, out.xres, out.yres, epsg)


def rasterize_table(table: GeometryTable, info: RasterInfo, *, values=None, fn: str = "last",
                    background=0, dtype: str = "float64", bands: np.ndarray | None = None,
                    n_bands: int | None = None, all_touched: bool = False,
                    context: _lib.Context | None = None, out: np.ndarray | None = None,
                    stats: dict | None = None, rows: tuple[int, int] | None = None) -> np.ndarray:
    """Burn ``table`` into a dense (bands, nrows, ncols) array of ``dtype``.

    values: None (burn 1), a scalar (FieldSource::Scalar) or a per-geometry
    array of ``dtype`` (FieldSource::Array).  bands: per-geometry band index
    (uint32) with ``n_bands`` bands, or None for one band.  rows: burn only
    the raster rows [r0, r1) (``rz_rasterize_rows``): the result is
    (bands, r1 - r0, ncols) and equals those rows of the whole burn.
    """
    lib = _lib.load()
    if dtype not in _lib.DTYPES:
        raise ValueError(f"Unsupported dtype {dtype!r}")
    if fn not in _lib.PIXEL_FNS:
        raise ValueError("Unknown pixel function")
    np_dt = np.dtype(dtype)
    ctx = context or _lib.default_context()
    nb = 1
    c_bands = None
    if bands is not None:
        bands = np.ascontiguousarray(bands, dtype=np.uint32)
        nb = int(n_bands if n_bands is not None else (int(bands.max()) + 1 if len(bands) else 1))
        c_bands = bands.ctypes.data
    flags = _lib.FLAG_ALL_TOUCHED if all_touched else 0
    vals_arr = None
    c_vals = None
    if values is not None:
        if np.isscalar(values) or (isinstance(values, np.ndarray) and values.ndim == 0):
            vals_arr = np.array([values], dtype=np_dt)
            flags |= _lib.FLAG_SCALAR_VALUE
        else:
            vals_arr = np.ascontiguousarray(values, dtype=np_dt)
            if len(vals_arr) != table.n_geoms:
                raise ValueError("Geometry and field lengths must match")
        c_vals = vals_arr.ctypes.data
    bg = np.array([background], dtype=np_dt)
    r0, r1 = (0, info.nrows) if rows is None else (int(rows[0]), int(rows[1]))
    if not 0 <= r0 <= r1 <= info.nrows:
        raise ValueError(f"rows {rows} are outside the raster's {info.nrows} rows")
    shape = (nb, r1 - r0, info.ncols)
    if out is None:
        out = np.empty(shape, dtype=np_dt)
    elif out.dtype != np_dt or out.shape != shape or not out.flags.c_contiguous:
        raise ValueError("out has the wrong dtype, shape or layout")
    g = table.c_view()
    ri = info.c_struct()
    st_c = _lib.RzStats()
    e = _lib.errbuf()
    with ctx.lock:
        if rows is None:
            st = lib.rz_rasterize(ctx.handle, ctypes.byref(g), c_vals, bg.ctypes.data, c_bands, nb,
                                  ctypes.byref(ri), _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags, out.ctypes.data,
                                  ctypes.byref(st_c), e, len(e))
        else:
            st = lib.rz_rasterize_rows(ctx.handle, ctypes.byref(g), c_vals, bg.ctypes.data, c_bands, nb,
                                       ctypes.byref(ri), r0, r1, _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags,
                                       out.ctypes.data, ctypes.byref(st_c), e, len(e))
    _lib.raise_for(st, e.value)
    if stats is not None:
        stats.update(st_c.as_dict())
    return out


class _SparseResult:
    """Owner of an engine sparse result (rz_sparse): numpy views of its
    columns keep it alive, and it is freed with the last of them."""

    def __init__(self, lib, handle):
        self._lib = lib
        self._h = handle

    def view(self, ptr: int, count: int, dtype) -> np.ndarray:
        dt = np.dtype(dtype)
        if count == 0 or not ptr:
            return np.empty(0, dtype=dt)
        nbytes = count * dt.itemsize
        # a subclass of the ctypes array type can carry the owner; numpy's
        # buffer keeps the ctypes object, and so the owner, alive
        buf_t = type("_SparseColumn", (ctypes.c_uint8 * nbytes,), {})
        buf = buf_t.from_address(ptr)
        buf._owner = self
        return np.frombuffer(buf, dtype=dt, count=count)

    def __del__(self):
        try:
            if self._h:
                self._lib.rz_sparse_free(self._h)
                self._h = None
        except Exception:
            pass


def copy_from_address(ptr: int, count: int, dtype) -> np.ndarray:
    """A numpy copy of `count` elements of `dtype` at host address `ptr`
    (any size: a view of the memory, then one copy)."""
    dt = np.dtype(dtype)
    if count == 0:
        return np.empty(0, dtype=dt)
    raw = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)), shape=(count * dt.itemsize,))
    return raw.view(dt).copy()


def rasterize_table_sparse(table: GeometryTable, info: RasterInfo, *, values=None, fn: str = "last",
                           dtype: str = "float64", bands: np.ndarray | None = None, n_bands: int | None = None,
                           all_touched: bool = False, context: _lib.Context | None = None,
                           stats: dict | None = None) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Burn ``table`` as COO triplets (the SparseArrayWriter stream,
    rust/src/encoding/writers.rs:86-131): returns (band_counts, rows, cols,
    values) with the triplets grouped by band in band order."""
    lib = _lib.load()
    if dtype not in _lib.DTYPES:
        raise ValueError(f"Unsupported dtype {dtype!r}")
    if fn not in _lib.PIXEL_FNS:
        raise ValueError("Unknown pixel function")
    np_dt = np.dtype(dtype)
    ctx = context or _lib.default_context()
    nb = 1
    c_bands = None
    if bands is not None:
        bands = np.ascontiguousarray(bands, dtype=np.uint32)
        nb = int(n_bands if n_bands is not None else (int(bands.max()) + 1 if len(bands) else 1))
        c_bands = bands.ctypes.data
    flags = _lib.FLAG_ALL_TOUCHED if all_touched else 0
    vals_arr = None
    c_vals = None
    if values is not None:
        if np.isscalar(values) or (isinstance(values, np.ndarray) and values.ndim == 0):
            vals_arr = np.array([values], dtype=np_dt)
            flags |= _lib.FLAG_SCALAR_VALUE
        else:
            vals_arr = np.ascontiguousarray(values, dtype=np_dt)
            if len(vals_arr) != table.n_geoms:
                raise ValueError("Geometry and field lengths must match")
        c_vals = vals_arr.ctypes.data
    g = table.c_view()
    ri = info.c_struct()
    st_c = _lib.RzStats()
    e = _lib.errbuf()
    h = ctypes.c_void_p()
    with ctx.lock:
        st = lib.rz_rasterize_sparse(ctx.handle, ctypes.byref(g), c_vals, c_bands, nb, ctypes.byref(ri),
                                     _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags, ctypes.byref(h),
                                     ctypes.byref(st_c), e, len(e))
    _lib.raise_for(st, e.value)
    owner = _SparseResult(lib, h)
    v = _lib.RzSparseView()
    lib.rz_sparse_view_get(h, ctypes.byref(v))
    n = int(v.count)
    band_counts = copy_from_address(v.band_counts, int(v.n_bands), np.uint64)
    # the triplet columns are views of the engine's arrays (no copy of the
    # stream); the result is freed when the last of them is collected
    rows = owner.view(v.rows, n, np.uint64)
    cols = owner.view(v.cols, n, np.uint64)
    vals = owner.view(v.values, n, np_dt)
    if stats is not None:
        stats.update(st_c.as_dict())
    return band_counts, rows, cols, vals


def sparse_build(band_counts, rows, cols, values, nrows: int, ncols: int, *, fn: str, background,
                 context: _lib.Context | None = None, out: np.ndarray | None = None,
                 stats: dict | None = None) -> np.ndarray:
    """Replay a COO triplet stream onto a (bands, nrows, ncols) raster of the
    values' dtype (``rz_sparse_build``; SparseArray::build_array,
    rust/src/encoding/arrays.rs:103-141): the raster starts at
    ``background`` and every triplet applies the pixel function ``fn`` to its
    pixel, each pixel's writes in stream order.  band_counts[b] triplets
    belong to band b, bands in order."""
    lib = _lib.load()
    if fn not in _lib.PIXEL_FNS:
        raise ValueError("Unknown pixel function")
    values = np.ascontiguousarray(values)
    dtype = values.dtype.name
    if dtype not in _lib.DTYPES:
        raise ValueError(f"Unsupported dtype {dtype!r}")
    counts = np.ascontiguousarray(band_counts, dtype=np.uint64)
    if counts.ndim != 1 or len(counts) == 0:
        raise ValueError("band_counts needs one count per band")
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    cols = np.ascontiguousarray(cols, dtype=np.uint64)
    n = int(counts.sum(dtype=np.uint64))
    if not len(rows) == len(cols) == len(values) == n:
        raise ValueError("rows, cols, values and the band counts disagree")
    shape = (len(counts), int(nrows), int(ncols))
    if out is None:
        out = np.empty(shape, dtype=values.dtype)
    elif out.dtype != values.dtype or out.shape != shape or not out.flags.c_contiguous:
        raise ValueError("out has the wrong dtype, shape or layout")
    bg = np.array([background], dtype=values.dtype)
    ctx = context or _lib.default_context()
    st_c = _lib.RzStats()
    e = _lib.errbuf()
    with ctx.lock:
        st = lib.rz_sparse_build(ctx.handle, counts.ctypes.data, len(counts), rows.ctypes.data, cols.ctypes.data,
                                 values.ctypes.data, shape[1], shape[2], _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype],
                                 bg.ctypes.data, 0, out.ctypes.data, ctypes.byref(st_c), e, len(e))
    _lib.raise_for(st, e.value)
    if stats is not None:
        stats.update(st_c.as_dict())
    return out



@dataclass
class BatchJob:
    """One job of ``rasterize_batch``: the arguments of one single-band burn.

    values: None (burn 1), a scalar, or a per-geometry array of the batch
    dtype (host arrays for ``rasterize_batch``; CUDA tensors of the dtype's
    bits for ``device.rasterize_batch_device``)."""

    table: Any  # GeometryTable, or device.DeviceTable for the device form
    info: RasterInfo
    values: Any = None
    fn: str = "last"
    background: Any = 0


def _job_struct(job: BatchJob, np_dt: np.dtype, keep: list, device: bool) -> _lib.RzJob:
    """The rz_job of one BatchJob; host buffers it points at go into `keep`."""
    if job.fn not in _lib.PIXEL_FNS:
        raise ValueError("Unknown pixel function")
    j = _lib.RzJob()
    j.geoms = job.table.c_view()
    j.info = job.info.c_struct()
    j.fn = _lib.PIXEL_FNS[job.fn]
    j.flags = 0
    bg = np.array([job.background], dtype=np_dt)
    keep.append(bg)
    j.background = bg.ctypes.data
    v = job.values
    if v is None:
        j.values = None
    elif np.isscalar(v) or (isinstance(v, np.ndarray) and v.ndim == 0):
        sv = np.array([v], dtype=np_dt)
        keep.append(sv)
        j.values = sv.ctypes.data
        j.flags |= _lib.FLAG_SCALAR_VALUE
    elif device:
        if v.numel() != job.table.table.n_geoms or v.element_size() != np_dt.itemsize:
            raise ValueError("Geometry and field lengths must match")
        j.values = v.data_ptr()
    else:
        arr = np.ascontiguousarray(v, dtype=np_dt)
        if len(arr) != job.table.n_geoms:
            raise ValueError("Geometry and field lengths must match")
        keep.append(arr)
        j.values = arr.ctypes.data
    return j


def run_batch(jobs: list[BatchJob], outs: list, out_ptrs: list[int], dtype: str, flags: int, wave_bytes: int,
              context: _lib.Context | None, stats: dict | None, device: bool) -> None:
    """One rz_rasterize_batch call over `jobs` writing `out_ptrs`."""
    lib = _lib.load()
    if dtype not in _lib.DTYPES:
        raise ValueError(f"Unsupported dtype {dtype!r}")
    np_dt = np.dtype(dtype)
    ctx = context or _lib.default_context()
    keep: list = [outs]
    arr = (_lib.RzJob * max(1, len(jobs)))()
    for i, job in enumerate(jobs):
        arr[i] = _job_struct(job, np_dt, keep, device)
        arr[i].out = out_ptrs[i]
    st = _lib.RzBatchStats()
    e = _lib.errbuf()
    with ctx.lock:
        rc = lib.rz_rasterize_batch(ctx.handle, arr, len(jobs), _lib.DTYPES[dtype], flags, int(wave_bytes),
                                    ctypes.byref(st), e, len(e))
    _lib.raise_for(rc, e.value)
    if stats is not None:
        stats.update(st.as_dict())


def rasterize_batch(jobs: list[BatchJob], *, dtype: str = "float64", all_touched: bool = False,
                    wave_bytes: int = 0, context: _lib.Context | None = None,
                    stats: dict | None = None) -> list[np.ndarray]:
    """Burn many independent jobs (host geometry tables) in one engine call
    (``rz_rasterize_batch``): one pass of the kernels per wave of jobs instead
    of one per job.  Returns one (1, nrows, ncols) array per job, each
    identical to ``rasterize_table`` of that job alone."""
    np_dt = np.dtype(dtype)
    outs = [np.empty((1, j.info.nrows, j.info.ncols), dtype=np_dt) for j in jobs]
    flags = _lib.FLAG_ALL_TOUCHED if all_touched else 0
    run_batch(jobs, outs, [o.ctypes.data for o in outs], dtype, flags, wave_bytes, context, stats, device=False)
    return outs
