"""Shared helpers of the test-suite (inputs, oracle / engine calls)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

import oracle
from rusterize_gb300 import geometry as G

GOLDEN = Path(__file__).resolve().parent / "golden"


def golden_inputs():
    spec = json.loads((GOLDEN / "golden_inputs.json").read_text())
    return spec["geoms"], np.array(spec["values"])


def explode(t: G.GeometryTable, values):
    """GeoDataFrame.explode().explode(): every polygon, linestring and point
    becomes its own geometry carrying its parent's value."""
    b = G.TableBuilder()
    vals = []
    for gi in range(t.n_geoms):
        for p in range(int(t.part_offsets[gi]), int(t.part_offsets[gi + 1])):
            kind = int(t.part_kind[p])
            rings = [(t.xy[int(t.vertex_offsets[r]):int(t.vertex_offsets[r + 1])], int(t.ring_flags[r]))
                     for r in range(int(t.ring_offsets[p]), int(t.ring_offsets[p + 1]))]
            if kind == G.POLYGON:
                cur = []
                for c, f in rings:
                    if f == 0 and cur:
                        b.add_part(kind, cur)
                        b.end_geometry()
                        vals.append(values[gi])
                        cur = []
                    cur.append((c, f))
                if cur:
                    b.add_part(kind, cur)
                    b.end_geometry()
                    vals.append(values[gi])
            elif kind == G.LINE:
                for c, f in rings:
                    b.add_part(kind, [(c, f)])
                    b.end_geometry()
                    vals.append(values[gi])
            else:
                for c, _ in rings:
                    for v in c:
                        b.add_part(kind, [(v[None], 0)])
                        b.end_geometry()
                        vals.append(values[gi])
    return b.build(), np.array(vals)


def grid_of(info) -> dict:
    if isinstance(info, dict):
        return info
    if isinstance(info, tuple):
        keys = ("nrows", "ncols", "xmin", "xmax", "ymin", "ymax", "xres", "yres")
        return dict(zip(keys, info))
    return dict(nrows=info.nrows, ncols=info.ncols, xmin=info.xmin, xmax=info.xmax, ymin=info.ymin, ymax=info.ymax,
                xres=info.xres, yres=info.yres)


def oracle_burn(table, grid, *, fn="last", values=None, background=0.0, dtype="float64", bands=None, n_bands=None,
                all_touched=False, counters=None):
    g = grid_of(grid)
    return oracle.rasterize(table, g["nrows"], g["ncols"], g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["xres"],
                            g["yres"], values=values, fn=fn, background=background, dtype=dtype, bands=bands,
                            n_bands=n_bands, all_touched=all_touched, counters=counters)


def gpu_burn(table, grid, *, fn="last", values=None, background=0.0, dtype="float64", bands=None, n_bands=None,
             all_touched=False, stats=None):
    from rusterize_gb300.engine import RasterInfo, rasterize_table

    g = grid_of(grid)
    info = RasterInfo(**g)
    return rasterize_table(table, info, values=values, fn=fn, background=background, dtype=dtype, bands=bands,
                           n_bands=n_bands, all_touched=all_touched, stats=stats)


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    """Bit-exact equality (NaN payloads included)."""
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    u = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    return np.array_equal(a.view(u), b.view(u))


def diff_report(a: np.ndarray, b: np.ndarray, limit: int = 8) -> str:
    u = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    bad = np.argwhere(a.view(u) != b.view(u))
    lines = [f"{len(bad)} differing pixels"]
    for idx in bad[:limit]:
        t = tuple(int(i) for i in idx)
        lines.append(f"  {t}: got {a[t]!r} expected {b[t]!r}")
    return "\n".join(lines)
