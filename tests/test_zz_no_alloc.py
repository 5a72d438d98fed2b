"""The allocation-free entry point, rz_rasterize_noalloc, against the regular
one, rz_rasterize, both called through the C ABI.

rz_rasterize_noalloc is for callers that cannot allocate device memory at the
moment they burn (serving loops whose device memory is budgeted up front and
must not grow or stall on cudaMalloc/cudaFree, plugin hosts that own every
allocation through their own pool): it takes device inputs and outputs and a stream, and takes all
of its scratch from one static device array of RZ_NOALLOC_SCRATCH_BYTES.
Its results must be bit-identical to rz_rasterize's, also on the second of
two calls in a row, whose scratch still holds the first call's contents.

The file is named so that pytest collects it last; it passes on its own in a
fresh process as well as after the rest of the suite."""

import ctypes

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import _lib
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth
from rusterize_gb300.device import DeviceTable, rasterize_device, upload

from _util import diff_report, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(dt, info, *, fn, background, dtype, values=None, bands=None, n_bands=1, out=None, scalar=None):
    """One rz_rasterize_noalloc call on torch's current stream; returns the
    output tensor (raw bytes) and the stats."""
    lib = _lib.load()
    np_dt = np.dtype(dtype)
    nbytes = n_bands * info.nrows * info.ncols * np_dt.itemsize
    if out is None:
        out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    bg = np.array([background], dtype=np_dt)
    flags = 0
    vals = None
    if scalar is not None:
        sv = np.array([scalar], dtype=np_dt)
        vals = sv.ctypes.data
        flags |= _lib.FLAG_SCALAR_VALUE
    elif values is not None:
        vals = values.data_ptr()
    g = dt.c_view()
    ri = info.c_struct()
    st = _lib.RzStats()
    e = _lib.errbuf()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.rz_rasterize_noalloc(stream, ctypes.byref(g), vals, bg.ctypes.data,
                                  bands.data_ptr() if bands is not None else None, n_bands, ctypes.byref(ri),
                                  _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags, out.data_ptr(), ctypes.byref(st),
                                  e, len(e))
    _lib.raise_for(rc, e.value)
    return out, st.as_dict()


def _as_array(t, dtype, shape):
    return t.cpu().numpy().view(np.uint8).view(np.dtype(dtype)).reshape(shape)


def _regular(dt, info, **kw):
    """The regular entry point, rz_rasterize, on the same device buffers."""
    return rasterize_device(dt, info, **kw)


def _mixed_job(seed, side=1500):
    """Polygons with holes, lines and points over a side x side raster."""
    rng = np.random.default_rng(seed)
    n = 3000
    cx, cy = rng.uniform(-20, side + 20, n), rng.uniform(-20, side + 20, n)
    polys = synth.star_polygons(rng, n, (3, 40), rng.uniform(2.0, 60.0, n), cx, cy,
                                n_holes=rng.integers(0, 3, n))
    lines = synth.random_walk_lines(rng, 1500, (2, 30), (1.0, 40.0), (0.0, 0.0, float(side), float(side)))
    points = synth.random_points(rng, 4000, (0.0, 0.0, float(side), float(side)))
    table = G.GeometryTable.concat([polys, lines, points])
    return table, rz.RasterInfo(nrows=side, ncols=side, xmin=0.0, xmax=float(side), ymin=0.0, ymax=float(side),
                                xres=1.0, yres=1.0)


@pytest.mark.parametrize("fn,dtype,background", [("sum", "float64", 0.0), ("count", "uint32", 0),
                                                 ("last", "int16", -1), ("min", "float32", np.nan)])
def test_noalloc_matches_rz_rasterize_twice(fn, dtype, background):
    table, info = _mixed_job(7)
    dt = DeviceTable.upload(table)
    rng = np.random.default_rng(11)
    vals = rng.integers(-5, 9, table.n_geoms).astype(dtype)
    d_vals = upload(vals)
    shape = (1, info.nrows, info.ncols)
    want = _as_array(_regular(dt, info, fn=fn, background=background, dtype=dtype, values=d_vals), dtype, shape)
    for call in range(2):
        out = torch.full((int(np.prod(shape)) * np.dtype(dtype).itemsize,), 0xA5 - call, dtype=torch.uint8,
                         device="cuda")
        out, st = _noalloc(dt, info, fn=fn, background=background, dtype=dtype, values=d_vals, out=out)
        got = _as_array(out, dtype, shape)
        assert same_bits(got, want), f"call {call + 1}: " + diff_report(got, want)
        assert st["spans"] > 0 and st["pixel_writes"] > 0


def test_noalloc_bands_and_non_square_pixels_twice():
    """Band routing and the deduplicated writes of non-square pixels, then a
    different job on the same scratch."""
    table, _ = _mixed_job(21, side=900)
    info = rz.RasterInfo(nrows=700, ncols=1100, xmin=0.0, xmax=900.0, ymin=0.0, ymax=900.0, xres=900.0 / 1100,
                         yres=900.0 / 700)
    dt = DeviceTable.upload(table)
    rng = np.random.default_rng(5)
    n_bands = 3
    bands = torch.from_numpy(rng.integers(0, n_bands, table.n_geoms).astype(np.int32)).cuda()
    vals = upload(rng.integers(1, 7, table.n_geoms).astype(np.uint16))
    shape = (n_bands, info.nrows, info.ncols)
    want = _as_array(_regular(dt, info, fn="sum", background=0, dtype="uint16", values=vals, bands=bands,
                              n_bands=n_bands), "uint16", shape)
    for call in range(2):
        out, _ = _noalloc(dt, info, fn="sum", background=0, dtype="uint16", values=vals, bands=bands,
                          n_bands=n_bands)
        got = _as_array(out, "uint16", shape)
        assert same_bits(got, want), f"call {call + 1}: " + diff_report(got, want)
    # a smaller job right after: nothing of the larger one may leak into it
    w = synth.plain_small(1001)
    info2 = rz.raster_info(w.table, res=w.res, extent=w.extent)
    dt2 = DeviceTable.upload(w.table)
    d_vals2 = upload(np.asarray(w.values, dtype=w.dtype)) if w.values is not None else None
    shape2 = (1, info2.nrows, info2.ncols)
    want2 = _as_array(_regular(dt2, info2, fn=w.fn, background=w.background, dtype=w.dtype, values=d_vals2),
                      w.dtype, shape2)
    for call in range(2):
        out, _ = _noalloc(dt2, info2, fn=w.fn, background=w.background, dtype=w.dtype, values=d_vals2)
        got = _as_array(out, w.dtype, shape2)
        assert same_bits(got, want2), f"call {call + 1}: " + diff_report(got, want2)


def test_noalloc_scalar_value():
    table, info = _mixed_job(3, side=600)
    dt = DeviceTable.upload(table)
    shape = (1, info.nrows, info.ncols)
    sv = np.array([2.5], dtype=np.float32)
    want = np.full(shape, np.nan, dtype=np.float32)
    lib = _lib.load()
    # the regular entry point with a host scalar (RZ_FLAG_SCALAR_VALUE)
    ctx = _lib.default_context()
    e = _lib.errbuf()
    st = _lib.RzStats()
    g = table.c_view()
    ri = info.c_struct()
    bg = np.array([np.nan], dtype=np.float32)
    with ctx.lock:
        rc = lib.rz_rasterize(ctx.handle, ctypes.byref(g), sv.ctypes.data, bg.ctypes.data, None, 1, ctypes.byref(ri),
                              _lib.PIXEL_FNS["sum"], _lib.DTYPES["float32"], _lib.FLAG_SCALAR_VALUE,
                              want.ctypes.data, ctypes.byref(st), e, len(e))
    _lib.raise_for(rc, e.value)
    for call in range(2):
        out, _ = _noalloc(dt, info, fn="sum", background=np.nan, dtype="float32", scalar=2.5)
        got = _as_array(out, "float32", shape)
        assert same_bits(got, want), f"call {call + 1}: " + diff_report(got, want)


def test_noalloc_rejects_jobs_beyond_its_scratch():
    limit = _lib.NOALLOC_SCRATCH_BYTES
    # bucket tables alone exceed the array: refused before any launch
    table, _ = _mixed_job(1, side=300)
    dt = DeviceTable.upload(table)
    big = rz.RasterInfo(nrows=100_000, ncols=100_000, xmin=0.0, xmax=300.0, ymin=0.0, ymax=300.0,
                        xres=0.003, yres=0.003)
    tiny = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError, match=str(limit)):
        _noalloc(dt, big, fn="count", background=0, dtype="uint8", out=tiny)
    # more spans than fit: 1000 full-width rectangles, 4 tiles x 2000 rows each
    b = G.TableBuilder()
    for i in range(1000):
        x0 = float(i % 7)
        G.add_polygon(b, np.array([[x0, 0.0], [2048.0 - x0, 0.0], [2048.0 - x0, 2000.0], [x0, 2000.0], [x0, 0.0]]))
    rect = b.build()
    info = rz.RasterInfo(nrows=2000, ncols=2048, xmin=0.0, xmax=2048.0, ymin=0.0, ymax=2000.0, xres=1.0, yres=1.0)
    drect = DeviceTable.upload(rect)
    with pytest.raises(ValueError, match="spans"):
        _noalloc(drect, info, fn="count", background=0, dtype="uint32")
    # the scratch is still usable afterwards
    want = _as_array(_regular(dt, rz.RasterInfo(nrows=300, ncols=300, xmin=0.0, xmax=300.0, ymin=0.0, ymax=300.0,
                                                xres=1.0, yres=1.0), fn="count", background=0, dtype="uint32"),
                     "uint32", (1, 300, 300))
    out, _ = _noalloc(dt, rz.RasterInfo(nrows=300, ncols=300, xmin=0.0, xmax=300.0, ymin=0.0, ymax=300.0, xres=1.0,
                                        yres=1.0), fn="count", background=0, dtype="uint32")
    assert same_bits(_as_array(out, "uint32", (1, 300, 300)), want)
