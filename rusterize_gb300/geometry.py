"""Flat geometry table (the engine's input layout) and its readers.

A top-level geometry is a run of *parts*; a part is a burn unit of
rusterize's ``Burn`` impls (rust/src/rasterization/burn_geometry.rs):

* ``POINT``   -- Point / MultiPoint: every vertex of the part is a point
* ``LINE``    -- LineString / MultiLineString: rings are linestrings whose
                 segments are pooled (one PixelCache, one "last segment")
* ``POLYGON`` -- Polygon / MultiPolygon: rings pooled into one even-odd set

A GeometryCollection is the concatenation of its members' parts.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import _lib

POINT, LINE, POLYGON = 0, 1, 2


@dataclass
class GeometryTable:
    part_offsets: np.ndarray    # uint64 [G+1]
    part_kind: np.ndarray       # uint8  [P]
    ring_offsets: np.ndarray    # uint64 [P+1]
    vertex_offsets: np.ndarray  # uint64 [R+1]
    ring_flags: np.ndarray      # uint8  [R]  (bit0: hole)
    xy: np.ndarray              # float64 [V, 2]

    def __post_init__(self):
        self.part_offsets = np.ascontiguousarray(self.part_offsets, dtype=np.uint64)
        self.part_kind = np.ascontiguousarray(self.part_kind, dtype=np.uint8)
        self.ring_offsets = np.ascontiguousarray(self.ring_offsets, dtype=np.uint64)
        self.vertex_offsets = np.ascontiguousarray(self.vertex_offsets, dtype=np.uint64)
        self.ring_flags = np.ascontiguousarray(self.ring_flags, dtype=np.uint8)
        self.xy = np.ascontiguousarray(np.asarray(self.xy, dtype=np.float64).reshape(-1, 2))

    @property
    def n_geoms(self) -> int:
        return len(self.part_offsets) - 1

    @property
    def n_parts(self) -> int:
        return len(self.part_kind)

    @property
    def n_rings(self) -> int:
        return len(self.ring_flags)

    @property
    def n_vertices(self) -> int:
        return len(self.xy)

    def __len__(self) -> int:
        return self.n_geoms

    def c_view(self) -> _lib.RzGeoms:
        g = _lib.RzGeoms()
        g.n_geoms, g.n_parts, g.n_rings, g.n_vertices = self.n_geoms, self.n_parts, self.n_rings, self.n_vertices
        g.part_offsets = self.part_offsets.ctypes.data
        g.part_kind = self.part_kind.ctypes.data
        g.ring_offsets = self.ring_offsets.ctypes.data
        g.vertex_offsets = self.vertex_offsets.ctypes.data
        g.ring_flags = self.ring_flags.ctypes.data
        g.xy = self.xy.ctypes.data
        return g

    def select(self, idx: Sequence[int]) -> "GeometryTable":
        """Sub-table of the given geometries (in the given order)."""
        idx = np.asarray(idx, dtype=np.int64).reshape(-1)

        def ranges(lo: np.ndarray, hi: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
            # the concatenation of arange(lo[i], hi[i]), and the offsets of its pieces
            n = (hi - lo).astype(np.int64)
            off = np.concatenate([[0], np.cumsum(n)]).astype(np.int64)
            flat = np.arange(int(off[-1]), dtype=np.int64) - np.repeat(off[:-1] - lo.astype(np.int64), n)
            return flat, off

        po, ro, vo = (a.astype(np.int64) for a in (self.part_offsets, self.ring_offsets, self.vertex_offsets))
        parts, new_po = ranges(po[idx], po[idx + 1])
        rings, new_ro = ranges(ro[parts], ro[parts + 1])
        verts, new_vo = ranges(vo[rings], vo[rings + 1])
        return GeometryTable(new_po.astype(np.uint64), self.part_kind[parts], new_ro.astype(np.uint64),
                             new_vo.astype(np.uint64), self.ring_flags[rings], self.xy[verts])

    def slice(self, g0: int, g1: int) -> "GeometryTable":
        """Sub-table of the contiguous geometries [g0, g1), offsets rebased."""
        p0, p1 = int(self.part_offsets[g0]), int(self.part_offsets[g1])
        r0, r1 = int(self.ring_offsets[p0]), int(self.ring_offsets[p1])
        v0, v1 = int(self.vertex_offsets[r0]), int(self.vertex_offsets[r1])
        return GeometryTable(self.part_offsets[g0:g1 + 1] - np.uint64(p0), self.part_kind[p0:p1],
                             self.ring_offsets[p0:p1 + 1] - np.uint64(r0), self.vertex_offsets[r0:r1 + 1] - np.uint64(v0),
                             self.ring_flags[r0:r1], self.xy[v0:v1])

    @staticmethod
    def concat(tables: Iterable["GeometryTable"]) -> "GeometryTable":
        tables = list(tables)
        po, pk, ro, vo, rf, xy = [np.zeros(1, np.uint64)], [], [np.zeros(1, np.uint64)], [np.zeros(1, np.uint64)], [], []
        P = R = V = 0
        for t in tables:
            po.append(t.part_offsets[1:] + np.uint64(P))
            ro.append(t.ring_offsets[1:] + np.uint64(R))
            vo.append(t.vertex_offsets[1:] + np.uint64(V))
            pk.append(t.part_kind)
            rf.append(t.ring_flags)
            xy.append(t.xy)
            P, R, V = P + t.n_parts, R + t.n_rings, V + t.n_vertices
        return GeometryTable(np.concatenate(po), np.concatenate(pk) if pk else np.zeros(0, np.uint8),
                             np.concatenate(ro), np.concatenate(vo),
                             np.concatenate(rf) if rf else np.zeros(0, np.uint8),
                             np.concatenate(xy) if xy else np.zeros((0, 2)))


class TableBuilder:
    """Incremental builder (used by tests and small programmatic inputs)."""

    def __init__(self):
        self.po, self.pk, self.ro, self.vo, self.rf = [0], [], [0], [0], []
        self.chunks: list[np.ndarray] = []
        self.nv = 0

    def add_part(self, kind: int, rings: Iterable[tuple[np.ndarray, int]]) -> None:
        for coords, flag in rings:
            c = np.asarray(coords, dtype=np.float64).reshape(-1, 2)
            self.chunks.append(c)
            self.nv += len(c)
            self.vo.append(self.nv)
            self.rf.append(flag)
        self.pk.append(kind)
        self.ro.append(len(self.rf))

    def end_geometry(self) -> None:
        self.po.append(len(self.pk))

    def build(self) -> GeometryTable:
        xy = np.concatenate(self.chunks) if self.chunks else np.zeros((0, 2))
        return GeometryTable(np.array(self.po, np.uint64), np.array(self.pk, np.uint8),
                             np.array(self.ro, np.uint64), np.array(self.vo, np.uint64),
                             np.array(self.rf, np.uint8), xy)


def _close(c: np.ndarray) -> np.ndarray:
    c = np.asarray(c, dtype=np.float64).reshape(-1, 2)
    if len(c) and not (c[0, 0] == c[-1, 0] and c[0, 1] == c[-1, 1]):
        c = np.vstack([c, c[:1]])
    return c


# convenience constructors: each appends ONE geometry
def add_point(b: TableBuilder, x: float, y: float) -> None:
    b.add_part(POINT, [(np.array([[x, y]]), 0)])
    b.end_geometry()


def add_multipoint(b: TableBuilder, pts) -> None:
    b.add_part(POINT, [(np.asarray(pts, dtype=np.float64), 0)])
    b.end_geometry()


def add_linestring(b: TableBuilder, coords) -> None:
    b.add_part(LINE, [(np.asarray(coords, dtype=np.float64), 0)])
    b.end_geometry()


def add_multilinestring(b: TableBuilder, lines) -> None:
    b.add_part(LINE, [(np.asarray(c, dtype=np.float64), 0) for c in lines])
    b.end_geometry()


def add_polygon(b: TableBuilder, exterior, holes=()) -> None:
    rings = [(_close(exterior), 0)] + [(_close(h), 1) for h in holes]
    b.add_part(POLYGON, rings)
    b.end_geometry()


def add_multipolygon(b: TableBuilder, polys) -> None:
    rings = []
    for poly in polys:
        ext, holes = poly[0], poly[1] if len(poly) > 1 else ()
        rings.append((_close(ext), 0))
        rings.extend((_close(h), 1) for h in holes)
    b.add_part(POLYGON, rings)
    b.end_geometry()


def _from_buffer(buf: ctypes.c_void_p) -> GeometryTable:
    lib = _lib.load()
    g = _lib.RzGeoms()
    lib.rz_geom_buffer_view(buf, ctypes.byref(g))

    def arr(p, n, dt, shape=None):
        if n == 0:
            return np.zeros(shape or 0, dt)
        ct = np.ctypeslib.as_array((ctypes.c_uint8 * (n * np.dtype(dt).itemsize)).from_address(p))
        out = ct.view(dt).copy()
        return out.reshape(shape) if shape else out

    t = GeometryTable(arr(g.part_offsets, g.n_geoms + 1, np.uint64), arr(g.part_kind, g.n_parts, np.uint8),
                      arr(g.ring_offsets, g.n_parts + 1, np.uint64), arr(g.vertex_offsets, g.n_rings + 1, np.uint64),
                      arr(g.ring_flags, g.n_rings, np.uint8),
                      arr(g.xy, 2 * g.n_vertices, np.float64, (g.n_vertices, 2)))
    lib.rz_geom_buffer_free(buf)
    return t


def from_wkt(texts: Sequence[str]) -> GeometryTable:
    """Parse WKT strings (python/src/geo/parse_geometry.rs:86-88,122-133)."""
    lib = _lib.load()
    enc = [t.encode() if isinstance(t, str) else bytes(t) for t in texts]
    n = len(enc)
    ptrs = (ctypes.c_char_p * n)(*enc)
    lens = (ctypes.c_size_t * n)(*[len(x) for x in enc])
    buf = ctypes.c_void_p()
    e = _lib.errbuf()
    st = lib.rz_parse_wkt(ptrs, lens, n, ctypes.byref(buf), e, len(e))
    _lib.raise_for(st, e.value)
    return _from_buffer(buf)


def from_wkb(blobs: Sequence[bytes]) -> GeometryTable:
    """Parse WKB blobs (python/src/geo/parse_geometry.rs:77-84,109-120)."""
    lib = _lib.load()
    # bytes objects are passed by pointer (no copy); their lengths bound the reads
    enc = [b if isinstance(b, bytes) else bytes(b) for b in blobs]
    n = len(enc)
    ptrs = (ctypes.c_char_p * n)(*enc)
    lens = (ctypes.c_size_t * n)(*[len(x) for x in enc])
    buf = ctypes.c_void_p()
    e = _lib.errbuf()
    st = lib.rz_parse_wkb(ptrs, lens, n, ctypes.byref(buf), e, len(e))
    _lib.raise_for(st, e.value)
    return _from_buffer(buf)
