"""Device-resident inputs and outputs (PyTorch is used only to own device
memory; the burn is the engine's).  Geometries uploaded once can be burned
many times without host<->device traffic."""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .engine import RasterInfo
from .geometry import GeometryTable


def _torch():
    import torch

    return torch


@dataclass
class DeviceTable:
    table: GeometryTable  # host copy (sizes)
    tensors: dict         # name -> torch CUDA tensor

    @classmethod
    def upload(cls, table: GeometryTable, device: int = 0) -> "DeviceTable":
        torch = _torch()
        dev = torch.device("cuda", device)

        def up(a):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

        t = {
            "part_offsets": up(table.part_offsets.view(np.int64)),
            "part_kind": up(table.part_kind),
            "ring_offsets": up(table.ring_offsets.view(np.int64)),
            "vertex_offsets": up(table.vertex_offsets.view(np.int64)),
            "ring_flags": up(table.ring_flags),
            "xy": up(table.xy),
        }
        return cls(table, t)

    def c_view(self) -> _lib.RzGeoms:
        g = _lib.RzGeoms()
        t = self.table
        g.n_geoms, g.n_parts, g.n_rings, g.n_vertices = t.n_geoms, t.n_parts, t.n_rings, t.n_vertices
        for name in ("part_offsets", "part_kind", "ring_offsets", "vertex_offsets", "ring_flags", "xy"):
            setattr(g, name, self.tensors[name].data_ptr())
        return g

    @property
    def nbytes(self) -> int:
        return sum(x.numel() * x.element_size() for x in self.tensors.values())


def upload(a: np.ndarray, device: int = 0):
    """Copy a numpy array to a CUDA tensor (unsigned types keep their bits)."""
    torch = _torch()
    a = np.ascontiguousarray(a)
    if a.dtype in (np.uint16, np.uint32, np.uint64):
        a = a.view({2: np.int16, 4: np.int32, 8: np.int64}[a.itemsize])
    return torch.from_numpy(a).to(torch.device("cuda", device))


def rasterize_device(dt: DeviceTable, info: RasterInfo, *, fn: str, background, dtype: str, values=None,
                     bands=None, n_bands: int = 1, out=None, context: _lib.Context | None = None,
                     stats: dict | None = None, rows: tuple[int, int] | None = None):
    """Burn a DeviceTable into a CUDA tensor (bands, nrows, ncols) of dtype.
    values: CUDA tensor of the output dtype's bits per geometry, or None (1);
    bands: CUDA int32 tensor of band indices, or None; rows: only the raster
    rows [r0, r1), into (bands, r1 - r0, ncols) (``rz_rasterize_rows``)."""
    torch = _torch()
    lib = _lib.load()
    ctx = context or _lib.default_context()
    np_dt = np.dtype(dtype)
    tdt = {"uint8": torch.uint8, "int8": torch.int8, "int16": torch.int16, "int32": torch.int32,
           "int64": torch.int64, "float32": torch.float32, "float64": torch.float64}.get(dtype)
    r0, r1 = (0, info.nrows) if rows is None else (int(rows[0]), int(rows[1]))
    if out is None:
        shape = (n_bands, r1 - r0, info.ncols)
        if tdt is None:  # unsigned wider than 8 bits: raw bytes
            out = torch.empty(int(np.prod(shape)) * np_dt.itemsize, dtype=torch.uint8, device=dt.tensors["xy"].device)
        else:
            out = torch.empty(shape, dtype=tdt, device=dt.tensors["xy"].device)
    bg = np.array([background], dtype=np_dt)
    g = dt.c_view()
    ri = info.c_struct()
    st = _lib.RzStats()
    e = _lib.errbuf()
    flags = _lib.FLAG_INPUT_DEVICE | _lib.FLAG_OUTPUT_DEVICE
    vals = values.data_ptr() if values is not None else None
    bptr = bands.data_ptr() if bands is not None else None
    with ctx.lock:
        if rows is None:
            rc = lib.rz_rasterize(ctx.handle, ctypes.byref(g), vals, bg.ctypes.data, bptr, n_bands,
                                  ctypes.byref(ri), _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags, out.data_ptr(),
                                  ctypes.byref(st), e, len(e))
        else:
            rc = lib.rz_rasterize_rows(ctx.handle, ctypes.byref(g), vals, bg.ctypes.data, bptr, n_bands,
                                       ctypes.byref(ri), r0, r1, _lib.PIXEL_FNS[fn], _lib.DTYPES[dtype], flags,
                                       out.data_ptr(), ctypes.byref(st), e, len(e))
    _lib.raise_for(rc, e.value)
    if stats is not None:
        stats.update(st.as_dict())
    return out


def rasterize_batch_device(jobs: list, *, dtype: str, outs: list | None = None, all_touched: bool = False,
                           wave_bytes: int = 0, context: _lib.Context | None = None, stats: dict | None = None):
    """``rz_rasterize_batch`` on device-resident jobs: each ``BatchJob``
    holds a DeviceTable and values as a CUDA tensor of the dtype's bits (or a
    scalar or None); the rasters are written into CUDA tensors (allocated
    when `outs` is None, one (1, nrows, ncols) raster per job)."""
    from .engine import run_batch

    torch = _torch()
    np_dt = np.dtype(dtype)
    if outs is None:
        outs = []
        for j in jobs:
            n = j.info.nrows * j.info.ncols
            outs.append(torch.empty(max(1, n * np_dt.itemsize), dtype=torch.uint8,
                                    device=j.table.tensors["xy"].device))
    flags = _lib.FLAG_INPUT_DEVICE | _lib.FLAG_OUTPUT_DEVICE | (_lib.FLAG_ALL_TOUCHED if all_touched else 0)
    run_batch(jobs, outs, [o.data_ptr() for o in outs], dtype, flags, wave_bytes, context, stats, device=True)
    return outs
