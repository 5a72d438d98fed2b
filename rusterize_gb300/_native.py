"""``_rusterize``: the native entry point under ``rusterize()``.

Mirrors python/src/rusterize.rs:127-184 (``_rusterize`` / rusterize_py_impl)
and python/src/geo/parse_geometry.rs:36-75 (ParsedGeometry::extract): the
same arguments, defaults, dispatch and error types, with the burn itself on
the GB300 engine through its C ABI.
"""

from __future__ import annotations

import math
import operator
from typing import Any

import numpy as np

from . import _lib
from ._dependencies import shapely
from ._lib import PanicException
from .engine import RasterInfo, raster_info, rasterize_table, rasterize_table_sparse
from .geometry import GeometryTable, from_wkb, from_wkt
from .sparse import SparseArray


def parse_geometry(obj: Any) -> GeometryTable:
    """ParsedGeometry::extract (parse_geometry.rs:36-75)."""
    if isinstance(obj, GeometryTable):
        return obj
    if hasattr(obj, "geom_type"):  # geopandas GeoSeries / GeoDataFrame
        return from_wkb(_to_wkb(obj))
    if isinstance(obj, list) or type(obj).__name__ == "ndarray":
        if len(obj) == 0:
            raise ValueError("No geometries found.")
        first = obj[0]
        if isinstance(first, (bytes, bytearray, memoryview)):
            return from_wkb(list(obj))
        if isinstance(first, str):
            return from_wkt([str(x) for x in obj])
        if hasattr(first, "geom_type"):
            return from_wkb(_to_wkb(obj))
        raise ValueError("Sequence must contain geometries as shapely Geometry, bytes (WKB), or string (WKT).")
    if type(obj).__name__ == "Series" and hasattr(obj, "dtype"):  # polars Series of WKB / WKT
        vals = [v for v in obj.to_list() if v is not None]
        if vals and isinstance(vals[0], (bytes, bytearray)):
            return from_wkb(vals)
        if vals and isinstance(vals[0], str):
            return from_wkt(vals)
        raise TypeError("Unsupported dtype for geometry column")
    raise TypeError("Unsupported geometry input type.")


def _to_wkb(obj: Any) -> list[bytes]:
    # shapely >= 2 (parse_geometry.rs:90-107)
    if not shapely.installed:
        raise ModuleNotFoundError("shapely must be installed to rasterize shapely geometries")
    if not str(shapely.__version__).startswith("2"):
        raise ValueError("Shapely version 2 required")
    return list(shapely.to_wkb(obj, output_dimension=2, include_srid=False, flavor="iso"))


def _extract(obj: Any, dtype: np.dtype) -> tuple[bool, Any]:
    """pyo3 ``obj.extract::<T>()`` for the raster dtypes."""
    if obj is None or isinstance(obj, (str, bytes, bytearray)):
        return False, None
    if dtype.kind in "ui":
        try:
            v = operator.index(obj)
        except TypeError:
            return False, None
        info = np.iinfo(dtype)
        if v < info.min or v > info.max:
            return False, None
        return True, v
    try:
        v = float(obj)
    except (TypeError, ValueError):
        return False, None
    with np.errstate(over="ignore"):
        return True, np.array(v, dtype=dtype)[()]


def _by_strings(col: Any) -> list[str | None]:
    """polars ``cast(DataType::String)`` of a `by` column."""
    out: list[str | None] = []
    for v in list(col):
        if v is None:
            out.append(None)
        elif isinstance(v, (bool, np.bool_)):
            out.append("true" if v else "false")
        elif isinstance(v, (int, np.integer)):
            out.append(str(int(v)))
        elif isinstance(v, (float, np.floating)):
            out.append(repr(float(v)))
        else:
            out.append(str(v))
    return out


def group_keys(by: list[str]) -> tuple[list[str], np.ndarray]:
    """rasterize.rs:198-205: bands are the sorted distinct keys (BTreeMap)."""
    names = sorted(set(by))
    index = {k: i for i, k in enumerate(names)}
    return names, np.fromiter((index[k] for k in by), dtype=np.uint32, count=len(by))


def _rusterize(geometry: Any, raw_raster_info: dict, pypixel_fn: str, pydf: Any = None, pyfield: str | None = None,
               pyby: str | None = None, pyburn: Any = None, pybackground: Any = None, pytouched: bool = False,
               pyencoding: str = "xarray", pydtype: str = "float64", *, context: _lib.Context | None = None,
               stats: dict | None = None):
    table = parse_geometry(geometry)
    try:
        info = raster_info(table, shape=raw_raster_info.get("shape"), res=raw_raster_info.get("resolution"),
                           extent=raw_raster_info.get("extent"), tap=bool(raw_raster_info.get("tap", False)),
                           epsg=raw_raster_info.get("epsg"))
    except ValueError as e:  # every RasterInfo error becomes RuntimeError (rusterize.rs:271)
        raise RuntimeError(str(e)) from None
    if pypixel_fn not in _lib.PIXEL_FNS:
        raise ValueError("Unknown pixel function")
    if pydtype not in _lib.DTYPES or pyencoding not in ("xarray", "numpy", "sparse"):
        raise PanicException("not implemented: Invalid dtype or encoding provided.")
    dt = np.dtype(pydtype)

    # rusterize.rs:50-53: background.extract::<T>().ok().unwrap_or_default()
    ok, bg = _extract(pybackground, dt)
    if not ok:
        bg = dt.type(0)

    # rusterize.rs:55-96: field column / burn / by
    field_col = by_col = None
    if pydf is not None:
        if pyfield is not None:
            field_col = pydf[pyfield]
        if pyby is not None:
            by_col = pydf[pyby]
    keep = None
    if field_col is not None:
        raw = list(field_col) if isinstance(field_col, (list, tuple)) else field_col
        arr = np.asarray(raw, dtype=object) if not isinstance(raw, np.ndarray) else raw
        if arr.dtype == object:
            keep = np.array([v is not None for v in arr], dtype=bool)
            values = np.array([v if v is not None else 0 for v in arr]).astype(dt)
        else:
            values = arr.astype(dt)
    elif pyburn is None:
        values = None
    else:
        ok, scalar = _extract(pyburn, dt)
        if ok:
            values = scalar
        elif isinstance(pyburn, np.ndarray) and pyburn.ndim == 1 and pyburn.dtype == dt:
            values = pyburn
        else:
            raise TypeError(f"'{type(pyburn).__name__}' object cannot be converted to 'PyArray<{dt.name}, Ix1>'")

    bands = None
    band_names = ["band_1"]
    if by_col is not None:
        by = _by_strings(by_col)
        if any(v is None for v in by):
            raise RuntimeError("Found nulls in `by` column. Consider droppping them.")
        band_names, bands = group_keys(by)

    # rasterize.rs:207-229 (raised through rusterize.rs:246 as RuntimeError)
    if values is not None and not np.isscalar(values) and getattr(values, "ndim", 1) != 0:
        if len(values) != table.n_geoms:
            raise RuntimeError("Geometry and field lengths must match")
    if bands is not None and len(bands) != table.n_geoms:
        raise RuntimeError("Geometry and by lengths must match")
    if keep is not None and not keep.all():  # null field values are not burned (rasterize.rs:188-192)
        idx = np.flatnonzero(keep)
        table = table.select(idx)
        values = values[idx]
        if bands is not None:
            bands = bands[idx]

    if pyencoding == "sparse":  # rusterize.rs:166-176 -> SparseArray (arrays.rs:62-101)
        band_counts, rows, cols, vals = rasterize_table_sparse(
            table, info, values=values, fn=pypixel_fn, dtype=pydtype, bands=bands, n_bands=len(band_names),
            all_touched=bool(pytouched), context=context, stats=stats)
        return SparseArray(band_names, band_counts, rows, cols, vals, info, pypixel_fn, bg)
    out = rasterize_table(table, info, values=values, fn=pypixel_fn, background=bg, dtype=pydtype, bands=bands,
                          n_bands=len(band_names), all_touched=bool(pytouched), context=context, stats=stats)
    if pyencoding == "xarray":
        return _to_xarray(out, info, band_names)
    return out


def _axis(start: float, end: float, step: float) -> np.ndarray:
    """ndarray's Array::range(start, end, step): ceil((end - start) / step)
    elements, element i = start + step * i (one rounding each for the product
    and the sum, no FMA)."""
    n = math.ceil((end - start) / step)
    return start + step * np.arange(max(n, 0), dtype=np.float64)


def make_coordinates(info: RasterInfo) -> tuple[np.ndarray, np.ndarray]:
    """Pixel-centre coordinates (y, x) of the raster: make_coordinates,
    python/src/geo/raster.rs:45-62 (y descends from ymax - yres / 2)."""
    y = _axis(info.ymax - info.yres / 2.0, info.ymax - float(info.nrows) * info.yres, -info.yres)
    x = _axis(info.xmin + info.xres / 2.0, info.xmin + float(info.ncols) * info.xres, info.xres)
    return y, x


def _to_xarray(data: np.ndarray, info: RasterInfo, band_names: list[str]):
    """build_xarray (python/src/encoding/xarray.rs:10-58): a DataArray with
    dims (bands, y, x), built with DataArray.from_dict from the same
    dictionary, and the EPSG code written as its CRS by rioxarray."""
    from ._dependencies import rioxarray
    from ._dependencies import xarray as xr

    rioxarray.load()  # registers the .rio accessor
    y, x = make_coordinates(info)
    spec = {
        "data": data,
        "dims": ["bands", "y", "x"],
        "coords": {"x": {"dims": "x", "data": x}, "y": {"dims": "y", "data": y},
                   "bands": {"dims": "bands", "data": list(band_names)}},
    }
    da = xr.DataArray.from_dict(spec)
    if info.epsg is not None:
        da = da.rio.write_crs(info.epsg)
    return da
