"""Host-side logic, CPU only: the C-ABI library loads and exports every
declared symbol, geometry readers, the raster-grid builder (checked against
the oracle's restatement), argument validation and band grouping."""

import ctypes
import re
import struct
from pathlib import Path

import numpy as np
import pytest

import oracle
import rusterize_gb300 as rz
from rusterize_gb300 import _lib
from rusterize_gb300 import geometry as G
from rusterize_gb300._native import _extract, group_keys

from _util import golden_inputs

HEADER = Path(__file__).resolve().parents[1] / "include" / "rusterize_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(rz_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.PROTOTYPES), "ctypes prototypes out of sync with the header"
    assert lib.rz_abi_version() == 1
    assert b"sm_103a" in lib.rz_build_info()


def test_dtype_sizes_and_pixel_fn_names():
    lib = _lib.load()
    assert [lib.rz_dtype_size(i) for i in range(10)] == [1, 2, 4, 8, 1, 2, 4, 8, 4, 8]
    assert lib.rz_dtype_size(99) == 0
    out = ctypes.c_int()
    e = _lib.errbuf()
    for name, code in _lib.PIXEL_FNS.items():
        assert lib.rz_pixel_fn_from_str(name.encode(), ctypes.byref(out), e, len(e)) == 0
        assert out.value == code
    assert lib.rz_pixel_fn_from_str(b"bogus", ctypes.byref(out), e, len(e)) == _lib.RZ_VALUE_ERROR
    assert e.value == b"Unknown pixel function"  # pixel_functions.rs:30


def test_wkt_reader_layout():
    t = G.from_wkt([
        "POINT (1 2)",
        "MULTIPOINT ((1 2), (3 4))",
        "MULTIPOINT (5 6, 7 8)",
        "LINESTRING (0 0, 1 1, 2 0)",
        "MULTILINESTRING ((0 0, 1 1), (2 2, 3 3))",
        "POLYGON ((0 0, 4 0, 4 4, 0 4, 0 0), (1 1, 2 1, 2 2, 1 1))",
        "POLYGON ((0 0, 4 0, 4 4))",  # unclosed: closed like geo-types Polygon::new
        "MULTIPOLYGON (((0 0, 1 0, 1 1, 0 0)), ((5 5, 6 5, 6 6, 5 5)))",
        "GEOMETRYCOLLECTION (POINT (1 1), GEOMETRYCOLLECTION (LINESTRING (0 0, 1 1)))",
        "POINT Z (1 2 3)",
        "polygon ((0 0, 1 0, 1 1, 0 0))",
    ])
    assert t.n_geoms == 11
    assert list(t.part_offsets) == [0, 1, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12]
    assert list(t.part_kind) == [0, 0, 0, 1, 1, 2, 2, 2, 0, 1, 0, 2]
    # polygon with hole: ring flags exterior, hole
    p = 5
    r0, r1 = t.ring_offsets[p], t.ring_offsets[p + 1]
    assert list(t.ring_flags[r0:r1]) == [0, 1]
    # unclosed ring got its closing vertex
    r = t.ring_offsets[6]
    v0, v1 = t.vertex_offsets[r], t.vertex_offsets[r + 1]
    assert v1 - v0 == 4 and np.array_equal(t.xy[v0], t.xy[v1 - 1])
    z = t.part_offsets[9]
    assert np.array_equal(t.xy[t.vertex_offsets[t.ring_offsets[z]]], [1, 2])


def test_wkt_errors():
    with pytest.raises(rz.PanicException, match="WKT"):
        G.from_wkt(["POLYGON ((0 0, 1 0"])
    with pytest.raises(rz.PanicException):
        G.from_wkt(["POINT EMPTY"])
    with pytest.raises(rz.PanicException):
        G.from_wkt(["CIRCLE (1 2)"])


def _wkb(kind, body, le=True):
    e = "<" if le else ">"
    return struct.pack(e[0] + "B", 1 if le else 0) + struct.pack(e + "I", kind) + body


def _pts(pts, le=True):
    e = "<" if le else ">"
    return b"".join(struct.pack(e + "dd", x, y) for x, y in pts)


def test_wkb_reader_matches_wkt():
    sq = [(0, 0), (4, 0), (4, 4), (0, 4), (0, 0)]
    hole = [(1, 1), (2, 1), (2, 2), (1, 1)]
    blobs = [
        _wkb(1, _pts([(1, 2)])),
        _wkb(3, struct.pack("<I", 2) + struct.pack("<I", 5) + _pts(sq) + struct.pack("<I", 4) + _pts(hole)),
        _wkb(2, struct.pack(">I", 3) + _pts([(0, 0), (1, 1), (2, 0)], le=False), le=False),
        _wkb(7, struct.pack("<I", 2) + _wkb(1, _pts([(1, 1)])) + _wkb(2, struct.pack("<I", 2) + _pts([(0, 0), (1, 1)]))),
        _wkb(1001, _pts([(1, 2)]) + struct.pack("<d", 3.0)),  # ISO POINT Z
        _wkb(6, struct.pack("<I", 1) + _wkb(3, struct.pack("<I", 1) + struct.pack("<I", 4) + _pts(hole))),
    ]
    a = G.from_wkb(blobs)
    b = G.from_wkt([
        "POINT (1 2)",
        "POLYGON ((0 0, 4 0, 4 4, 0 4, 0 0), (1 1, 2 1, 2 2, 1 1))",
        "LINESTRING (0 0, 1 1, 2 0)",
        "GEOMETRYCOLLECTION (POINT (1 1), LINESTRING (0 0, 1 1))",
        "POINT (1 2)",
        "MULTIPOLYGON (((1 1, 2 1, 2 2, 1 1)))",
    ])
    for f in ("part_offsets", "part_kind", "ring_offsets", "vertex_offsets", "ring_flags", "xy"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_wkb_empty_point_is_dropped():
    # try_to_geometry() -> None is skipped (parse_geometry.rs:113-115)
    blobs = [_wkb(1, _pts([(np.nan, np.nan)])), _wkb(1, _pts([(3, 4)]))]
    t = G.from_wkb(blobs)
    assert t.n_geoms == 1
    with pytest.raises(ValueError, match="Could not parse geometry"):
        G.from_wkb(blobs[:1])
    with pytest.raises(rz.PanicException, match="WKB"):
        G.from_wkb([b"\x01\x03\x00"])


@pytest.mark.parametrize("seed", range(40))
def test_raster_info_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 6))
    b = G.TableBuilder()
    for _ in range(n):
        c = rng.uniform(-500, 500, 2)
        G.add_polygon(b, c + rng.uniform(-50, 50, (int(rng.integers(3, 9)), 2)))
    if seed % 3 == 0:
        G.add_point(b, *rng.uniform(-600, 600, 2))
    t = b.build()
    mode = seed % 4
    kw = {}
    if mode == 0:
        kw = dict(res=tuple(rng.uniform(0.1, 7, 2)))
    elif mode == 1:
        kw = dict(shape=tuple(int(x) for x in rng.integers(1, 500, 2)))
    elif mode == 2:
        kw = dict(res=tuple(rng.uniform(0.3, 3, 2)), extent=(-100.0, -50.0, 250.5, 80.25))
    else:
        kw = dict(res=tuple(rng.uniform(0.3, 3, 2)), tap=True)
    got = rz.raster_info(t, **kw)
    exp = oracle.raster_info(t, **kw)
    assert (got.nrows, got.ncols, got.xmin, got.xmax, got.ymin, got.ymax, got.xres, got.yres) == exp


def test_raster_info_errors_and_extent_uses_exteriors():
    b = G.TableBuilder()
    G.add_polygon(b, [(0, 0), (4, 0), (4, 4), (0, 4)], holes=[[(-10, -10), (20, -10), (20, 20)]])
    t = b.build()
    info = rz.raster_info(t, res=(1, 1))
    assert (info.nrows, info.ncols) == (5, 5)  # the hole does not widen the bounding box
    with pytest.raises(ValueError, match="Must set at least one"):
        rz.raster_info(t)
    with pytest.raises(ValueError, match="mutually exclusive"):
        rz.raster_info(t, res=(1, 1), shape=(3, 3))
    with pytest.raises(ValueError, match="Resolution values must be > 0."):
        rz.raster_info(t, res=(0, 1))
    with pytest.raises(ValueError, match="Unspecified extent"):
        rz.raster_info(t, res=(1, 1), extent=(0, 0, 0, 0))
    assert rz.raster_info(t, res=(1, 1), extent=(-0.0, 0, 0, 0)).nrows == 0
    empty = G.from_wkt(["GEOMETRYCOLLECTION EMPTY"])
    with pytest.raises(RuntimeError, match="Cannot infer bounding box"):
        rz.raster_info(empty, res=(1, 1))


def test_background_and_burn_extraction():
    # python/src/rusterize.rs:50-53 extract::<T>().ok().unwrap_or_default()
    assert _extract(np.nan, np.dtype("uint8"))[0] is False
    assert _extract(-1, np.dtype("uint8"))[0] is False
    assert _extract(300, np.dtype("uint8"))[0] is False
    assert _extract(2.5, np.dtype("int32"))[0] is False
    assert _extract(7, np.dtype("int8")) == (True, 7)
    assert _extract(True, np.dtype("uint8")) == (True, 1)
    ok, v = _extract(1e40, np.dtype("float32"))
    assert ok and np.isinf(v)
    assert _extract(None, np.dtype("float64"))[0] is False


def test_group_keys_sorted_like_btreemap():
    # rasterize.rs:306-313 and the lexicographic order of string keys
    names, idx = group_keys(["b", "a", "b"])
    assert names == ["a", "b"] and list(idx) == [1, 0, 1]
    names, idx = group_keys([str(c) for c in (0, 1, 10, 2, 15, 9)])
    assert names == ["0", "1", "10", "15", "2", "9"]


class TestTypeChecks:
    # python/test/test_many.py:46-71
    @pytest.mark.parametrize(
        "kwargs, match",
        [
            ({"data": "not_a_dataframe", "res": (1, 1)}, "`data` must be either geopandas"),
            ({"like": "not_an_xarray", "res": (1, 1), "encoding": "numpy"}, "`like` must be a xarray.DataArray"),
            ({"res": "1x1"}, "`resolution` must be a tuple or list"),
            ({"out_shape": "100x100"}, "`out_shape` must be a tuple or list"),
            ({"extent": "0,0,10,10"}, "`extent` must be a tuple or list"),
            ({"field": 123}, "`field` must be a string"),
            ({"by": 123}, "`by` must be a string"),
            ({"burn": "hot"}, "`burn` must be an integer, float"),
            ({"fun": 1}, "`pixel_fn` must be one of"),
            ({"background": "black"}, "`background` must be integer, float, or None"),
            ({"encoding": 1}, "`encoding` must be one of 'xarray'"),
            ({"all_touched": "yes"}, "`all_touched` must be a boolean"),
            ({"tap": "yes"}, "`tap` must be a boolean"),
            ({"dtype": 64}, "`dtype` must be a one of"),
        ],
    )
    def test_type_errors(self, kwargs, match):
        geoms, _ = golden_inputs()
        args = {"data": geoms, "res": (1, 1), "encoding": "numpy"}
        args.update(kwargs)
        with pytest.raises(TypeError, match=match):
            rz.rusterize(**args)


class TestArguments:
    # python/test/test_many.py:115-163
    def setup_method(self):
        self.geoms, _ = golden_inputs()

    def test_mutually_exclusive_field_burn(self):
        with pytest.raises(ValueError, match="Only one of `field` or `burn` can be specified"):
            rz.rusterize(self.geoms, res=(1, 1), field="value", burn=5, encoding="numpy")

    def test_burn_array_length_mismatch(self):
        with pytest.raises(ValueError, match=re.escape("If `burn` is a `numpy.ndarray`, it must have the same length as `data`.")):
            rz.rusterize(self.geoms, res=(1, 1), burn=np.array([1, 2]), encoding="numpy")

    def test_missing_spatial_metadata_error(self):
        with pytest.raises(ValueError, match="One of `res`, `out_shape`, or `extent` must be provided"):
            rz.rusterize(self.geoms, encoding="numpy")

    def test_invalid_resolution_error(self):
        with pytest.raises(ValueError, match="`res` must be 2 positive numbers"):
            rz.rusterize(self.geoms, res=(-1, 1), encoding="numpy")

    def test_invalid_shape_error(self):
        with pytest.raises(ValueError, match="`out_shape` must be 2 positive integers"):
            rz.rusterize(self.geoms, out_shape=(-1, 1), encoding="numpy")

    def test_invalid_extent_error1(self):
        with pytest.raises(ValueError, match="Must also specify `res` or `out_shape` with extent."):
            rz.rusterize(self.geoms, extent=(1, 2, 3, 4), encoding="numpy")

    def test_invalid_extent_error2(self):
        with pytest.raises(ValueError, match=re.escape("`extent` must be a tuple or list of (xmin, ymin, xmax, ymax).")):
            rz.rusterize(self.geoms, res=(1, 1), extent=(0, 0, 0, 0), encoding="numpy")

    def test_res_and_shape_exclusive(self):
        with pytest.raises(ValueError, match="mutually exclusive"):
            rz.rusterize(self.geoms, res=(1, 1), out_shape=(3, 3), encoding="numpy")

    def test_bad_encoding(self):
        with pytest.raises(ValueError, match="`encoding` must be one of"):
            rz.rusterize(self.geoms, res=(1, 1), encoding="bogus")

    def test_xarray_encoding_missing(self):
        # xarray/rioxarray are not installed here (test_many.py:101-104)
        if rz._dependencies._xarray_available():
            pytest.skip("xarray installed")
        with pytest.raises(ModuleNotFoundError, match="`xarray` and `rioxarray` must be installed"):
            rz.rusterize(self.geoms, res=(1, 1), encoding="xarray")

    def test_empty_sequence(self):
        with pytest.raises(ValueError, match="No geometries found."):
            rz._rusterize([], {"resolution": (1, 1), "tap": False}, "last", pyencoding="numpy")

    def test_bad_sequence_items(self):
        with pytest.raises(ValueError, match="Sequence must contain geometries"):
            rz._rusterize([1, 2], {"resolution": (1, 1), "tap": False}, "last", pyencoding="numpy")

    def test_unknown_pixel_fn(self):
        with pytest.raises(ValueError, match="Unknown pixel function"):
            rz._rusterize(self.geoms, {"resolution": (1, 1), "tap": False}, "bogus", pyencoding="numpy")

    def test_raster_info_errors_are_runtime_errors(self):
        # python/src/rusterize.rs:269-271
        with pytest.raises(RuntimeError, match="Resolution values must be > 0."):
            rz._rusterize(self.geoms, {"resolution": (0, 1), "tap": False}, "last", pyencoding="numpy")
