"""The xarray encoding without xarray: pixel-centre coordinates and the
DataArray specification, against a restatement of the reference's
make_coordinates (python/src/geo/raster.rs:45-62) and build_xarray
(python/src/encoding/xarray.rs:10-58).

ndarray's Array::range(a, b, step) has ceil((b - a) / step) elements and
element i is a + step * i; the restatement below computes both with Python
floats, one element at a time."""

from __future__ import annotations

import math
import types

import numpy as np
import pytest

from rusterize_gb300 import _dependencies, _native
from rusterize_gb300.engine import RasterInfo


def _range_loop(a: float, b: float, step: float) -> list[float]:
    n = math.ceil((b - a) / step)
    return [a + step * float(i) for i in range(max(n, 0))]


INFOS = [
    RasterInfo(1000, 1000, 0.0, 1000.0, 0.0, 1000.0, 1.0, 1.0),
    RasterInfo(131, 361, 2.0, 363.5, -7.25, 123.75, 1.0, 1.0),
    RasterInfo(47, 319, 523.9, 1127.1, -42.3, 45.6, 1.89, 1.87),
    RasterInfo(7, 3, -0.1, 0.2, -0.7, 0.0, 0.1, 0.1),
    RasterInfo(20000, 20000, 0.0, 20000.0, 0.0, 20000.0, 1.0, 1.0),
    RasterInfo(3, 5, 1e6 + 0.3, 1e6 + 0.3 + 5 * 1 / 3, 2e6, 2e6 + 3 * 1 / 7, 1 / 3, 1 / 7),
]


@pytest.mark.parametrize("info", INFOS)
def test_coordinates_match_ndarray_range(info):
    y, x = _native.make_coordinates(info)
    want_y = _range_loop(info.ymax - info.yres / 2.0, info.ymax - info.nrows * info.yres, -info.yres)
    want_x = _range_loop(info.xmin + info.xres / 2.0, info.xmin + info.ncols * info.xres, info.xres)
    assert y.dtype == np.float64 and x.dtype == np.float64
    assert y.tolist() == want_y and x.tolist() == want_x
    assert len(y) == info.nrows and len(x) == info.ncols


def test_random_grids_have_one_coordinate_per_pixel():
    rng = np.random.default_rng(7)
    for _ in range(2000):
        nrows, ncols = (int(v) for v in rng.integers(1, 5000, 2))
        xres, yres = (float(v) for v in np.exp(rng.uniform(-6, 6, 2)))
        xmin, ymin = (float(v) for v in rng.uniform(-1e6, 1e6, 2))
        info = RasterInfo(nrows, ncols, xmin, xmin + ncols * xres, ymin, ymin + nrows * yres, xres, yres)
        y, x = _native.make_coordinates(info)
        assert y.tolist() == _range_loop(info.ymax - yres / 2.0, info.ymax - nrows * yres, -yres)
        assert x.tolist() == _range_loop(xmin + xres / 2.0, xmin + ncols * xres, xres)


def test_dataarray_spec_with_stand_in_module(monkeypatch):
    seen = {}

    class _Rio:
        def __init__(self, da):
            self.da = da

        def write_crs(self, crs):
            seen["crs"] = crs
            return self.da

    class DataArray:
        @classmethod
        def from_dict(cls, d):
            seen["spec"] = d
            obj = cls()
            obj.rio = _Rio(obj)
            return obj

    fake_xr = types.SimpleNamespace(DataArray=DataArray)
    fake_rio = types.SimpleNamespace(load=lambda: None)
    monkeypatch.setattr(_dependencies, "xarray", fake_xr)
    monkeypatch.setattr(_dependencies, "rioxarray", fake_rio)
    info = RasterInfo(4, 6, 10.0, 16.0, 20.0, 24.0, 1.0, 1.0, epsg=32633)
    data = np.zeros((2, 4, 6), np.float32)
    _native._to_xarray(data, info, ["a", "b"])
    spec = seen["spec"]
    assert spec["dims"] == ["bands", "y", "x"]
    assert spec["data"] is data
    assert spec["coords"]["bands"] == {"dims": "bands", "data": ["a", "b"]}
    assert spec["coords"]["y"]["dims"] == "y" and spec["coords"]["x"]["dims"] == "x"
    assert spec["coords"]["y"]["data"].tolist() == [23.5, 22.5, 21.5, 20.5]
    assert spec["coords"]["x"]["data"].tolist() == [10.5, 11.5, 12.5, 13.5, 14.5, 15.5]
    assert seen["crs"] == 32633


def test_optional_module_raises_when_missing():
    m = _dependencies.OptionalModule("rusterize_gb300_no_such_module")
    assert not m.installed
    with pytest.raises(ModuleNotFoundError, match="rusterize_gb300_no_such_module"):
        m.DataArray  # noqa: B018
