"""ctypes binding of ``librusterize_gb300.so`` (C ABI: include/rusterize_gb300.h).

There is no CPU fallback: if the library is missing, or no GPU is usable,
calls raise instead of silently computing something else.
"""

from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_size_t, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

from ._build import lib_path

RZ_OK, RZ_VALUE_ERROR, RZ_RUNTIME_ERROR, RZ_PARSE_ERROR = 0, 1, 2, 3
RZ_CUDA_ERROR, RZ_NO_DEVICE, RZ_OUT_OF_MEMORY, RZ_INVALID_ARGUMENT = 4, 5, 6, 7

FLAG_ALL_TOUCHED = 1 << 0
FLAG_INPUT_DEVICE = 1 << 1
FLAG_OUTPUT_DEVICE = 1 << 2
FLAG_SCALAR_VALUE = 1 << 3
FLAG_NO_TIMING = 1 << 4

RI_SHAPE, RI_RES, RI_EXTENT, RI_TAP = 1, 2, 4, 8

NOALLOC_SCRATCH_BYTES = 64 * 1024 * 1024  # RZ_NOALLOC_SCRATCH_BYTES

# rz_dtype codes, in the order of python/src/rusterize.rs:171-182
DTYPES = {
    "uint8": 0, "uint16": 1, "uint32": 2, "uint64": 3,
    "int8": 4, "int16": 5, "int32": 6, "int64": 7,
    "float32": 8, "float64": 9,
}
PIXEL_FNS = {"sum": 0, "first": 1, "last": 2, "min": 3, "max": 4, "count": 5, "any": 6}


class PanicException(BaseException):
    """Raised where the reference panics (pyo3 turns a Rust panic into
    ``pyo3_runtime.PanicException``, a BaseException): malformed WKT/WKB
    (python/src/geo/parse_geometry.rs:78-87) and an unsupported dtype or
    encoding (python/src/rusterize.rs:151)."""


class EngineError(RuntimeError):
    """A CUDA-level failure of the GB300 engine."""


class NoDeviceError(EngineError):
    """No usable CUDA device: the engine has no CPU fallback."""


class RzGeoms(ctypes.Structure):
    _fields_ = [
        ("n_geoms", c_uint64), ("n_parts", c_uint64), ("n_rings", c_uint64), ("n_vertices", c_uint64),
        ("part_offsets", c_void_p), ("part_kind", c_void_p), ("ring_offsets", c_void_p),
        ("vertex_offsets", c_void_p), ("ring_flags", c_void_p), ("xy", c_void_p),
    ]


class RzRasterInfo(ctypes.Structure):
    _fields_ = [
        ("nrows", c_uint64), ("ncols", c_uint64),
        ("xmin", c_double), ("xmax", c_double), ("ymin", c_double), ("ymax", c_double),
        ("xres", c_double), ("yres", c_double), ("epsg", c_int32), ("_pad", c_int32),
    ]


class RzStats(ctypes.Structure):
    _fields_ = [
        ("edges", c_uint64), ("crossings", c_uint64), ("spans", c_uint64), ("pixel_writes", c_uint64),
        ("buckets", c_uint64), ("big_buckets", c_uint64), ("out_bytes", c_uint64),
        ("reruns", c_uint32), ("kernel_launches", c_uint32),
        ("ms_h2d", c_float), ("ms_prep", c_float), ("ms_spans", c_float), ("ms_bucket", c_float),
        ("ms_fill", c_float), ("ms_d2h", c_float), ("ms_device_total", c_float), ("ms_host_total", c_float),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class RzJob(ctypes.Structure):
    _fields_ = [
        ("geoms", RzGeoms), ("values", c_void_p), ("background", c_void_p), ("info", RzRasterInfo),
        ("fn", c_int), ("flags", c_uint32), ("out", c_void_p),
    ]


class RzBatchStats(ctypes.Structure):
    _fields_ = [
        ("jobs", c_uint64), ("waves", c_uint64), ("edges", c_uint64), ("records", c_uint64),
        ("pixel_writes", c_uint64), ("out_bytes", c_uint64), ("kernel_launches", c_uint32), ("reruns", c_uint32),
        ("ms_device_total", c_float), ("ms_host_total", c_float),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class RzTuning(ctypes.Structure):
    """rz_tuning: the schedule of a context (0 fields: defaults)."""

    _fields_ = [
        ("narrow_chunk", c_uint32), ("narrow_blocks_per_sm", c_uint32), ("wide_blocks_per_sm", c_uint32),
        ("rows_per_window", c_uint32), ("narrow_max_words", c_uint32), ("fill_sort_max", c_uint32),
        ("scatter_blocks_per_sm", c_uint32), ("line_blocks_per_sm", c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}

    @classmethod
    def from_dict(cls, d: dict) -> "RzTuning":
        t = cls()
        for name, _ in cls._fields_:
            setattr(t, name, int(d.get(name, 0)))
        return t


class RzSparseView(ctypes.Structure):
    _fields_ = [
        ("count", c_uint64), ("n_bands", c_uint32), ("dtype", c_int),
        ("band_counts", c_void_p), ("rows", c_void_p), ("cols", c_void_p), ("values", c_void_p),
    ]


# exported symbols and their prototypes (restype, argtypes)
PROTOTYPES = {
    "rz_abi_version": (c_int, []),
    "rz_build_info": (c_char_p, []),
    "rz_dtype_size": (c_size_t, [c_int]),
    "rz_pixel_fn_from_str": (c_int, [c_char_p, POINTER(c_int), c_char_p, c_size_t]),
    "rz_parse_wkt": (c_int, [POINTER(c_char_p), POINTER(c_size_t), c_size_t, POINTER(c_void_p), c_char_p, c_size_t]),
    "rz_parse_wkb": (c_int, [POINTER(c_char_p), POINTER(c_size_t), c_size_t, POINTER(c_void_p), c_char_p, c_size_t]),
    "rz_geom_buffer_view": (c_int, [c_void_p, POINTER(RzGeoms)]),
    "rz_geom_buffer_free": (None, [c_void_p]),
    "rz_raster_info_build": (c_int, [POINTER(RzGeoms), c_uint32, POINTER(c_uint64), POINTER(c_double),
                                     POINTER(c_double), c_int32, POINTER(RzRasterInfo), c_char_p, c_size_t]),
    "rz_context_create": (c_int, [c_int, POINTER(c_void_p), c_char_p, c_size_t]),
    "rz_context_destroy": (None, [c_void_p]),
    "rz_context_trim": (c_int, [c_void_p]),
    "rz_context_synchronize": (c_int, [c_void_p, c_char_p, c_size_t]),
    "rz_context_stream": (c_void_p, [c_void_p]),
    "rz_context_get_tuning": (c_int, [c_void_p, POINTER(RzTuning)]),
    "rz_context_set_tuning": (c_int, [c_void_p, POINTER(RzTuning), c_char_p, c_size_t]),
    "rz_rasterize": (c_int, [c_void_p, POINTER(RzGeoms), c_void_p, c_void_p, c_void_p, c_uint32,
                             POINTER(RzRasterInfo), c_int, c_int, c_uint32, c_void_p, POINTER(RzStats),
                             c_char_p, c_size_t]),
    "rz_rasterize_rows": (c_int, [c_void_p, POINTER(RzGeoms), c_void_p, c_void_p, c_void_p, c_uint32,
                                  POINTER(RzRasterInfo), c_uint64, c_uint64, c_int, c_int, c_uint32, c_void_p,
                                  POINTER(RzStats), c_char_p, c_size_t]),
    "rz_rasterize_noalloc": (c_int, [c_void_p, POINTER(RzGeoms), c_void_p, c_void_p, c_void_p, c_uint32,
                                     POINTER(RzRasterInfo), c_int, c_int, c_uint32, c_void_p, POINTER(RzStats),
                                     c_char_p, c_size_t]),
    "rz_rasterize_sparse": (c_int, [c_void_p, POINTER(RzGeoms), c_void_p, c_void_p, c_uint32, POINTER(RzRasterInfo),
                                    c_int, c_int, c_uint32, POINTER(c_void_p), POINTER(RzStats), c_char_p, c_size_t]),
    "rz_sparse_view_get": (c_int, [c_void_p, POINTER(RzSparseView)]),
    "rz_sparse_free": (None, [c_void_p]),
    "rz_sparse_build": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_uint64, c_uint64,
                                c_int, c_int, c_void_p, c_uint32, c_void_p, POINTER(RzStats), c_char_p, c_size_t]),
    "rz_rasterize_batch": (c_int, [c_void_p, POINTER(RzJob), c_size_t, c_int, c_uint32, c_uint64,
                                   POINTER(RzBatchStats), c_char_p, c_size_t]),
}

_lib = None
_lib_lock = threading.Lock()


def load() -> ctypes.CDLL:
    """Load the engine library (building it first if the sources are newer)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            path = Path(os.environ.get("RUSTERIZE_GB300_LIB", lib_path()))
            if "RUSTERIZE_GB300_LIB" not in os.environ:
                from ._build import build, needs_build

                if needs_build():
                    path = build()
            lib = ctypes.CDLL(str(path))
            for name, (res, args) in PROTOTYPES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def raise_for(status: int, msg: bytes | str, *, runtime_for_value: bool = False) -> None:
    if status == RZ_OK:
        return
    text = msg.decode() if isinstance(msg, (bytes, bytearray)) else str(msg)
    if status == RZ_VALUE_ERROR:
        raise (RuntimeError if runtime_for_value else ValueError)(text)
    if status == RZ_RUNTIME_ERROR:
        raise RuntimeError(text)
    if status == RZ_PARSE_ERROR:
        raise PanicException(text)
    if status == RZ_NO_DEVICE:
        raise NoDeviceError(text)
    if status == RZ_OUT_OF_MEMORY:
        raise MemoryError(text)
    if status == RZ_INVALID_ARGUMENT:
        raise ValueError(text)
    raise EngineError(text)


def errbuf() -> ctypes.Array:
    return ctypes.create_string_buffer(1024)


def ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


class Context:
    """One engine context: a CUDA stream plus a cached device scratch arena."""

    def __init__(self, device: int = 0):
        lib = load()
        h = c_void_p()
        e = errbuf()
        st = lib.rz_context_create(device, ctypes.byref(h), e, len(e))
        raise_for(st, e.value)
        self._h = h
        self._lib = lib
        self.device = device
        self.lock = threading.Lock()

    @property
    def handle(self) -> c_void_p:
        return self._h

    def synchronize(self) -> None:
        e = errbuf()
        raise_for(self._lib.rz_context_synchronize(self._h, e, len(e)), e.value)

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self._lib.rz_context_stream(self._h) or 0)

    def trim(self) -> None:
        self._lib.rz_context_trim(self._h)

    @property
    def tuning(self) -> dict:
        """The schedule in force (rz_context_get_tuning), defaults filled in."""
        t = RzTuning()
        raise_for(self._lib.rz_context_get_tuning(self._h, ctypes.byref(t)), b"rz_context_get_tuning failed")
        return t.as_dict()

    def set_tuning(self, tuning: dict | None) -> None:
        """Set the schedule (rz_context_set_tuning); None restores the defaults.
        Fields left out (or 0) take their defaults."""
        e = errbuf()
        with self.lock:
            if tuning is None:
                st = self._lib.rz_context_set_tuning(self._h, None, e, len(e))
            else:
                t = RzTuning.from_dict(tuning)
                st = self._lib.rz_context_set_tuning(self._h, ctypes.byref(t), e, len(e))
        raise_for(st, e.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.rz_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_contexts: dict[int, Context] = {}
_ctx_lock = threading.Lock()


def default_context(device: int | None = None) -> Context:
    if device is None:
        device = int(os.environ.get("RUSTERIZE_GB300_DEVICE", "0"))
    with _ctx_lock:
        ctx = _contexts.get(device)
        if ctx is None:
            ctx = Context(device)
            _contexts[device] = ctx
        return ctx
