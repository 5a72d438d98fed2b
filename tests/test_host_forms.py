"""Host-side pieces of the sparse and batched forms, without a GPU: the
SparseArray's reference-format repr and size hint (pyarray.rs:77-127) and
triplet columns, and the rz_job structs a batch call passes to the engine."""

import ctypes

import numpy as np
import pytest

from rusterize_gb300 import _lib
from rusterize_gb300 import geometry as G
from rusterize_gb300.engine import BatchJob, RasterInfo, _job_struct
from rusterize_gb300.sparse import SparseArray


def _info(nrows, ncols, epsg=None):
    return RasterInfo(nrows=nrows, ncols=ncols, xmin=0.0, xmax=float(ncols), ymin=0.0, ymax=float(nrows), xres=1.0,
                      yres=1.0, epsg=epsg)


def _sparse(n_bands, nrows, ncols, dtype="float64", epsg=None):
    names = [f"b{i}" for i in range(n_bands)]
    counts = np.array([2] + [1] * (n_bands - 1), dtype=np.uint64)
    n = int(counts.sum())
    return SparseArray(names, counts, np.arange(n, dtype=np.uint64), np.zeros(n, dtype=np.uint64),
                       np.ones(n, dtype=dtype), _info(nrows, ncols, epsg), "sum", 0)


@pytest.mark.parametrize("shape,dtype,hint", [
    ((1, 10, 10), "uint8", "100 bytes"),
    ((1, 10, 100), "float64", "8.00 KB"),
    ((3, 100, 100), "float64", "240.00 KB"),
    ((1, 1000, 1000), "float32", "4.00 MB"),
    ((2, 20000, 20000), "float64", "6.40 GB"),
])
def test_sparse_size_hint_and_repr(shape, dtype, hint):
    sp = _sparse(shape[0], shape[1], shape[2], dtype)
    assert sp.size_hint() == hint
    r = repr(sp)
    assert r.startswith(f"SparseArray:\n- Shape: {shape}\n- Extent: (0.0, 0.0, {float(shape[2])}, {float(shape[1])})\n")
    assert r.endswith(f"- Resolution: (1.0, 1.0)\n- EPSG: None\n- Estimated size: {hint}")
    assert "EPSG: 4326" in repr(_sparse(1, 5, 5, epsg=4326))


def test_sparse_triplet_columns():
    one = _sparse(1, 4, 4).triplets()
    assert list(one) == ["row", "col", "values"]  # no band column for one band (arrays.rs:188-200)
    three = _sparse(3, 4, 4).triplets()
    assert list(three) == ["band", "row", "col", "values"]
    assert three["band"].tolist() == [1, 1, 2, 3]  # 1-based, repeated by the band counts


def test_batch_job_structs():
    b = G.TableBuilder()
    G.add_polygon(b, np.array([[0.0, 0.0], [4.0, 0.0], [4.0, 4.0], [0.0, 0.0]]))
    G.add_point(b, 1.0, 1.0)
    t = b.build()
    keep = []
    j = _job_struct(BatchJob(t, _info(8, 8), values=np.array([2.0, 3.0]), fn="max", background=np.nan),
                    np.dtype("float32"), keep, device=False)
    assert j.fn == _lib.PIXEL_FNS["max"] and j.flags == 0 and j.geoms.n_geoms == 2 and j.info.ncols == 8
    vals = np.ctypeslib.as_array(ctypes.cast(j.values, ctypes.POINTER(ctypes.c_float)), (2,))
    assert vals.tolist() == [2.0, 3.0]
    assert np.isnan(ctypes.cast(j.background, ctypes.POINTER(ctypes.c_float))[0])
    s = _job_struct(BatchJob(t, _info(8, 8), values=5, fn="sum"), np.dtype("uint8"), keep, device=False)
    assert s.flags == _lib.FLAG_SCALAR_VALUE and ctypes.cast(s.values, ctypes.POINTER(ctypes.c_uint8))[0] == 5
    n = _job_struct(BatchJob(t, _info(8, 8)), np.dtype("int16"), keep, device=False)
    assert not n.values and n.fn == _lib.PIXEL_FNS["last"]
    with pytest.raises(ValueError, match="lengths"):
        _job_struct(BatchJob(t, _info(8, 8), values=np.ones(3)), np.dtype("float64"), keep, device=False)
    with pytest.raises(ValueError, match="pixel function"):
        _job_struct(BatchJob(t, _info(8, 8), fn="mean"), np.dtype("float64"), keep, device=False)
    assert ctypes.sizeof(_lib.RzJob) == 80 + 8 + 8 + 72 + 4 + 4 + 8


def test_copy_from_address_any_dtype_and_empty():
    from rusterize_gb300.engine import copy_from_address

    for dt in ("uint8", "int16", "float32", "uint64", "float64"):
        a = (np.arange(1000) * 3 - 7).astype(dt)
        b = copy_from_address(a.ctypes.data, len(a), dt)
        assert b.dtype == np.dtype(dt) and np.array_equal(a, b) and b.ctypes.data != a.ctypes.data
    assert copy_from_address(0, 0, "float64").shape == (0,)


def test_sparse_result_views_free_the_engine_result_with_the_last_view():
    import gc

    from rusterize_gb300.engine import _SparseResult

    freed = []

    class _FakeLib:
        def rz_sparse_free(self, h):
            freed.append(h)

    backing = (ctypes.c_uint64 * 10)(*range(10))
    owner = _SparseResult(_FakeLib(), 1234)
    a = owner.view(ctypes.addressof(backing), 10, np.uint64)
    b = owner.view(ctypes.addressof(backing), 5, np.float64)
    assert owner.view(0, 0, np.uint8).shape == (0,)
    del owner
    gc.collect()
    assert freed == [] and a.tolist() == list(range(10)) and len(b) == 5
    del a
    gc.collect()
    assert freed == []
    del b
    gc.collect()
    assert freed == [1234]
