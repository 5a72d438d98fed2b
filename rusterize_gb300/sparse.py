"""The sparse (COO) encoding: rusterize's SparseArray
(rust/src/encoding/arrays.rs:62-209, exposed to Python by
python/src/encoding/pyarray.rs:48-146).

The triplets come from the GPU engine (``rz_rasterize_sparse``): one
(row, col, value) triplet per pixel write, grouped by band in band order and
within a band by geometry in input order -- the reference's stream, except
that the triplets of one geometry come row by row, left to right.  Every
pixel therefore sees the same sequence of writes.  ``to_numpy`` is the
reference's ``build_array``: the stored triplets replayed onto a background
raster with the pixel function, on the GPU (``rz_sparse_build``), which
equals the dense encoding of the same burn bit for bit.
"""

from __future__ import annotations

import numpy as np

from .engine import RasterInfo


class SparseArray:
    """A sparse array in COOrdinate format storing the band/row/col value
    triplets of all burned geometries."""

    def __init__(self, band_names, band_counts, rows, cols, values, info: RasterInfo, fn: str, background):
        self._band_names = list(band_names)
        self._offsets = np.asarray(band_counts, dtype=np.uint64)
        if len(self._offsets) != len(self._band_names):
            raise ValueError("one triplet count per band is needed")
        self.rows = np.ascontiguousarray(rows, dtype=np.uint64)
        self.cols = np.ascontiguousarray(cols, dtype=np.uint64)
        self.values = np.ascontiguousarray(values)
        if not len(self.rows) == len(self.cols) == len(self.values) == int(self._offsets.sum()):
            raise ValueError("rows, cols, values and the band counts disagree")
        self._info = info
        self._fn = fn  # the pixel function and background the triplets replay with
        self._background = background

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
        nbytes = self.values.dtype.itemsize * nb * nr * nc
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

    def to_numpy(self, *, context=None, stats: dict | None = None) -> np.ndarray:
        """build_array (arrays.rs:103-141): the stored triplets replayed onto
        a background raster with the pixel function, each pixel's writes in
        stream order (on the GPU: ``rz_sparse_build``)."""
        from .engine import sparse_build

        return sparse_build(self._offsets, self.rows, self.cols, self.values, self._info.nrows, self._info.ncols,
                            fn=self._fn, background=self._background, context=context, stats=stats)

    def to_xarray(self):
        from ._native import _to_xarray

        return _to_xarray(self.to_numpy(), self._info, self._band_names)

    def to_frame(self):
        """A polars DataFrame of the triplets (arrays.rs:179-209); needs polars."""
        from ._dependencies import polars as pl

        return pl.DataFrame(self.triplets())
