"""rusterize_gb300 -- GB300-native (sm_103a) engine behind rusterize's
``rusterize()`` call.

``rusterize()`` keeps the reference's signature, defaults, validation and
error messages (python/python/rusterize/__init__.py:83-356); the burn runs
on the GPU through ``librusterize_gb300.so`` (C ABI in
include/rusterize_gb300.h).  There is no CPU fallback.
"""

from __future__ import annotations

from types import NoneType
from typing import Any

import numpy as np

from ._dependencies import (
    _check_for_geopandas,
    _check_for_polars_st,
    _polars_available,
    _xarray_available,
)
from ._dependencies import geopandas as gpd
from ._dependencies import polars as pl
from ._dependencies import xarray as xr
from ._lib import Context, EngineError, NoDeviceError, PanicException, default_context
from ._native import _rusterize, group_keys, parse_geometry
from .engine import BatchJob, RasterInfo, raster_info, rasterize_batch, rasterize_table, rasterize_table_sparse
from .geometry import GeometryTable, TableBuilder, from_wkb, from_wkt
from .sparse import SparseArray

__version__ = "0.1.0"

__all__ = [
    "rusterize", "_rusterize", "GeometryTable", "TableBuilder", "from_wkt", "from_wkb", "RasterInfo",
    "raster_info", "rasterize_table", "rasterize_table_sparse", "rasterize_batch", "BatchJob", "SparseArray",
    "group_keys", "parse_geometry", "Context", "default_context",
    "PanicException", "EngineError", "NoDeviceError",
]


def rusterize(
    data: Any,
    like: Any = None,
    res: tuple | list | None = None,
    out_shape: tuple | list | None = None,
    extent: tuple | list | None = None,
    field: str | None = None,
    by: str | None = None,
    burn: int | float | np.ndarray | None = None,
    fun: str = "last",
    background: int | float | None = np.nan,
    encoding: str = "xarray",
    all_touched: bool = False,
    tap: bool = False,
    dtype: str = "float64",
):
    """Rasterize geometries on the GPU.

    Parameters and semantics are those of the reference ``rusterize()``:
    data (geopandas.GeoDataFrame / GeoSeries, polars DataFrame with a
    "geometry" column, or a list / numpy array of WKT strings, WKB bytes or
    shapely geometries; additionally a :class:`GeometryTable`), like, res,
    out_shape, extent, field, by, burn, fun (sum, first, last, min, max,
    count, any), background, encoding ("xarray", "numpy", "sparse"),
    all_touched, tap and dtype.
    """
    if isinstance(data, (list, np.ndarray, GeometryTable)):
        data_type = "raw"
    elif _check_for_geopandas(data) and isinstance(data, gpd.GeoSeries):
        if data.empty:
            raise ValueError("Input data is empty.")
        data_type = "geoseries"
    elif _check_for_geopandas(data) and isinstance(data, gpd.GeoDataFrame):
        if data.empty:
            raise ValueError("Input data is empty.")
        data_type = "geopandas"
    elif _check_for_polars_st(data) and isinstance(data, pl.DataFrame):
        if data.is_empty():
            raise ValueError("Input data is empty.")
        data_type = "polars"
    else:
        raise TypeError(
            "`data` must be either geopandas.GeoDataFrame, geopandas.GeoSeries, polars.DataFrame, list, or numpy.ndarray"
        )

    if not isinstance(res, (tuple, list, NoneType)):
        raise TypeError("`resolution` must be a tuple or list of (xres, yres).")
    if not isinstance(out_shape, (tuple, list, NoneType)):
        raise TypeError("`out_shape` must be a tuple or list of (nrows, ncols).")
    if not isinstance(extent, (tuple, list, NoneType)):
        raise TypeError("`extent` must be a tuple or list of (xmin, ymin, xmax, ymax).")
    if not isinstance(field, (str, NoneType)):
        raise TypeError("`field` must be a string column name.")
    if not isinstance(by, (str, NoneType)):
        raise TypeError("`by` must be a string column name.")
    if not isinstance(burn, (int, float, np.ndarray, NoneType)):
        raise TypeError("`burn` must be an integer, float, or a numpy.ndarray.")
    if not isinstance(fun, str):
        raise TypeError("`pixel_fn` must be one of sum, first, last, min, max, count, or any.")
    if not isinstance(background, (int, float, NoneType)):
        raise TypeError("`background` must be integer, float, or None.")
    if not isinstance(encoding, str):
        raise TypeError("`encoding` must be one of 'xarray', 'numpy', or 'sparse'.")
    if not isinstance(all_touched, bool):
        raise TypeError("`all_touched` must be a boolean.")
    if not isinstance(tap, bool):
        raise TypeError("`tap` must be a boolean.")
    if not isinstance(dtype, str):
        raise TypeError(
            "`dtype` must be a one of 'uint8', 'uint16', 'uint32', 'uint64', 'int8', 'int16', 'int32', 'int64', 'float32', 'float64'"
        )
    if encoding not in ["xarray", "numpy", "sparse"]:
        raise ValueError("`encoding` must be one of `xarray`, 'numpy', or `sparse`.")
    if encoding == "xarray" and not _xarray_available():
        raise ModuleNotFoundError(
            "`xarray` and `rioxarray` must be installed if encoding is `xarray`. Install with `pip install xarray rioxarray`."
        )
    if field and burn is not None:
        raise ValueError("Only one of `field` or `burn` can be specified.")
    if isinstance(burn, np.ndarray) and burn.size != len(data):
        raise ValueError("If `burn` is a `numpy.ndarray`, it must have the same length as `data`.")

    _bounds = None
    _res = None
    _shape = None
    if like is not None:
        if not (_xarray_available() and isinstance(like, (xr.DataArray, xr.Dataset))):
            raise TypeError("`like` must be a xarray.DataArray or xarray.Dataset")
        if any((res, out_shape, extent)):
            raise ValueError("`like` is mutually exclusive with `res`, `out_shape`, and `extent`.")
        if not hasattr(like, "rio"):
            raise AttributeError("The `like` object must have a 'rio' accessor.")
        try:
            _shape = like.squeeze().shape
            _bounds = like.rio.bounds()
        except Exception as e:
            raise AttributeError("No spatial dimension found for like object") from e
    else:
        if not res and not out_shape and not extent:
            raise ValueError("One of `res`, `out_shape`, or `extent` must be provided.")
        if res and out_shape:
            raise ValueError("`res` and `out_shape` are mutually exclusive; provide only one.")
        if extent:
            if not res and not out_shape:
                raise ValueError("Must also specify `res` or `out_shape` with extent.")
            if len(extent) != 4 or all(e == 0 for e in extent):
                raise ValueError("`extent` must be a tuple or list of (xmin, ymin, xmax, ymax).")
            _bounds = extent
        if res:
            if len(res) != 2 or any(r <= 0 for r in res) or any(not isinstance(r, (int, float)) for r in res):
                raise ValueError("`res` must be 2 positive numbers.")
            _res = res
        if out_shape:
            if len(out_shape) != 2 or any(s <= 0 for s in out_shape) or any(not isinstance(s, int) for s in out_shape):
                raise ValueError("`out_shape` must be 2 positive integers.")
            _shape = out_shape

    cols = list(set([col for col in (field, by) if col and col != "geometry"]))
    df = None
    epsg = None
    match data_type:
        case "geopandas":
            epsg = data.crs.to_epsg() if data.crs else None
            if cols:
                if field and not by:
                    try:
                        burn = data[field].to_numpy()
                        field = None
                    except KeyError as e:
                        raise KeyError("Column not found in GeoDataFrame.") from e
                else:
                    if not _polars_available():
                        raise ModuleNotFoundError("polars must be installed when data is geopandas.GeoDataFrame.")
                    try:
                        df = pl.from_pandas(data[cols])
                    except KeyError as e:
                        raise KeyError("Column not found in GeoDataFrame.") from e
            geometries = data.geometry
        case "polars":
            try:
                srid = data.select(pl.col("geometry").first().st.srid()).item()
            except pl.exceptions.ColumnNotFoundError as e:
                raise ValueError("If `polars.DataFrame`, a 'geometry' column is expected.") from e
            epsg = None if srid == 0 else srid
            if cols:
                try:
                    df = data.select(pl.col([*cols, "geometry"]))
                except pl.exceptions.ColumnNotFoundError as e:
                    raise KeyError("Column not found in polars DataFrame.") from e
            geometries = data.select(pl.col("geometry")).to_series()
        case "geoseries":
            geometries = data.geometry
            burn = burn if burn is not None else data.index.to_numpy()
            try:
                epsg = data.crs.to_epsg()
            except AttributeError:
                pass
        case _:
            geometries = data

    if isinstance(burn, np.ndarray) and burn.dtype != dtype:
        burn = np.ascontiguousarray(burn, dtype=dtype)

    raw_raster_info = {"shape": _shape, "extent": _bounds, "resolution": _res, "tap": tap, "epsg": epsg}
    return _rusterize(geometries, raw_raster_info, fun, df, field, by, burn, background, all_touched, encoding, dtype)
