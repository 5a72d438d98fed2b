"""The sparse (COO) encoding: rusterize's SparseArray
(rust/src/encoding/arrays.rs:62-209, exposed to Python by
python/src/encoding/pyarray.rs:48-146).

The triplets come from the GPU engine (``rz_rasterize_sparse``): one
(row, col, value) triplet per pixel write, grouped by band in band order and
within a band by geometry in input order -- the reference's stream, except
that the triplets of one geometry come row by row, left to right.  Every
pixel therefore sees the same sequence of writes, and ``to_numpy`` (the
reference's ``build_array``: the writes replayed onto a background raster
with the pixel function) equals the dense encoding bit for bit; it is
materialised by the same engine.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .engine import RasterInfo


@dataclass
class _Burn:
    """What the dense replay needs: the inputs of the sparse call."""

    table: object
    values: object
    fn: str
    dtype: str
    background: object
    bands: np.ndarray | None
    all_touched: bool


class SparseArray:
    """A sparse array in COOrdinate format storing the band/row/col value
    triplets of all burned geometries."""

    def __init__(self, band_names, band_counts, rows, cols, values, info: RasterInfo, burn: _Burn):
        self._band_names = list(band_names)
        self._offsets = np.asarray(band_counts, dtype=np.uint64)
        self.rows = rows
        self.cols = cols
        self.values = values
        self._info = info
        self._burn = burn

    # ---- spatial information (arrays.rs:150-176) ----
    def band_names(self) -> list[str]:
        return list(self._band_names)

    def shape(self) -> tuple[int, int, int]:
        return (len(self._band_names), self._info.nrows, self._info.ncols)

    def extent(self) -> tuple[float, float, float, float]:
        return (self._info.xmin, self._info.ymin, self._info.xmax, self._info.ymax)

    def resolution(self) -> tuple[float, float]:
        return (self._info.xres, self._info.yres)

    def epsg(self):
        return self._info.epsg

    def size_hint(self) -> str:
        """Estimated size of the materialized dense array (pyarray.rs:77-91)."""
        nb, nr, nc = self.shape()
        nbytes = np.dtype(self._burn.dtype).itemsize * nb * nr * nc
        if nbytes < 1000:
            return f"{nbytes} bytes"
        f = np.float32(nbytes)  # the size is formatted from an f32 there
        if nbytes < 1_000_000:
            return f"{float(f / np.float32(1000.0)):.2f} KB"
        if nbytes < 1_000_000_000:
            return f"{float(f / np.float32(1_000_000.0)):.2f} MB"
        return f"{float(f / np.float32(1_000_000_000.0)):.2f} GB"

    def __repr__(self) -> str:
        epsg = self.epsg()
        return (f"SparseArray:\n- Shape: {self.shape()}\n- Extent: {self.extent()}\n"
                f"- Resolution: {self.resolution()}\n- EPSG: {'None' if epsg is None else epsg}\n"
                f"- Estimated size: {self.size_hint()}")

    # ---- materialisation ----
    def triplets(self) -> dict[str, np.ndarray]:
        """The COO columns as numpy arrays: band (1-based, only with several
        bands), row, col, values -- the columns of ``to_frame``."""
        out: dict[str, np.ndarray] = {}
        if len(self._offsets) > 1:
            out["band"] = np.repeat(np.arange(1, len(self._offsets) + 1, dtype=np.uint64),
                                    self._offsets.astype(np.int64))
        out["row"] = self.rows
        out["col"] = self.cols
        out["values"] = self.values
        return out

    def to_numpy(self) -> np.ndarray:
        """build_array (arrays.rs:103-141): the writes replayed onto a
        background raster with the pixel function."""
        from .engine import rasterize_table

        b = self._burn
        return rasterize_table(b.table, self._info, values=b.values, fn=b.fn, background=b.background,
                               dtype=b.dtype, bands=b.bands, n_bands=len(self._band_names),
                               all_touched=b.all_touched)

    def to_xarray(self):
        from ._native import _to_xarray

        return _to_xarray(self.to_numpy(), self._info, self._band_names)

    def to_frame(self):
        """A polars DataFrame of the triplets (arrays.rs:179-209); needs polars."""
        from ._dependencies import polars as pl

        return pl.DataFrame(self.triplets())
