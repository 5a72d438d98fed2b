"""Known-answer tests of the reference, restated as (inputs, expected).

Sources (ttrotto/rusterize):
  R/rusterize/tests/testthat/test-boundary.R, test-geometry.R  (4x4 grids)
  rust/src/rasterization/burn_geometry.rs:284-378              (10x10 grids)
  rust/src/rasterize.rs:251-304
R matrices are column-major; the expectations below are written row-major
(row 0 = top = ymax), which is the layout of the dense raster.
"""

from __future__ import annotations

import numpy as np

from rusterize_gb300 import geometry as G

GRID4 = dict(nrows=4, ncols=4, xmin=0.0, xmax=4.0, ymin=0.0, ymax=4.0, xres=1.0, yres=1.0)
GRID10 = dict(nrows=10, ncols=10, xmin=0.0, xmax=10.0, ymin=0.0, ymax=10.0, xres=1.0, yres=1.0)


def sq(x0, y0, x1, y1):
    return [(x0, y0), (x1, y0), (x1, y1), (x0, y1), (x0, y0)]


def table(*adders):
    b = G.TableBuilder()
    for add in adders:
        add(b)
    return b.build()


def poly(ext, holes=()):
    return lambda b: G.add_polygon(b, ext, holes)


def mpoly(*polys):
    return lambda b: G.add_multipolygon(b, [[p] for p in polys])


def point(x, y):
    return lambda b: G.add_point(b, x, y)


def mpoint(pts):
    return lambda b: G.add_multipoint(b, pts)


def line(coords):
    return lambda b: G.add_linestring(b, coords)


def mline(lines):
    return lambda b: G.add_multilinestring(b, lines)


def _m(rows):
    return np.array(rows, dtype=np.float64)


# (name, table, grid, kwargs, expected (bands, rows, cols) or a checker)
def r_kats():
    full = table(poly(sq(0, 0, 4, 4)))
    two = table(poly(sq(0, 0, 4, 4)), poly(sq(0, 0, 4, 4)))
    halves = table(poly(sq(0, 0, 2, 4)), poly(sq(2, 0, 4, 4)))
    left_right = _m([[10, 10, 20, 20]] * 4)
    kats = [
        # test-boundary.R:53-56
        ("full_coverage", full, GRID4, dict(fn="last", values=7.0, background=0.0), np.full((1, 4, 4), 7.0)),
        # test-boundary.R:58-62
        ("partial_coverage", table(poly(sq(0, 0, 2, 2))), GRID4, dict(fn="last", values=9.0, background=0.0),
         _m([[0, 0, 0, 0], [0, 0, 0, 0], [9, 9, 0, 0], [9, 9, 0, 0]])[None]),
        # test-boundary.R:64-68
        ("field_per_geometry", halves, GRID4, dict(fn="last", values=np.array([10.0, 20.0]), background=0.0),
         left_right[None]),
        # test-boundary.R:70-82
        ("sum", two, GRID4, dict(fn="sum", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 12.0)),
        ("min", two, GRID4, dict(fn="min", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 5.0)),
        ("max", two, GRID4, dict(fn="max", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 7.0)),
        ("first", two, GRID4, dict(fn="first", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 5.0)),
        ("last", two, GRID4, dict(fn="last", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 7.0)),
        ("count", two, GRID4, dict(fn="count", values=np.array([1.0, 1.0]), background=0.0), np.full((1, 4, 4), 2.0)),
        # test-geometry.R:3-7
        ("any", two, GRID4, dict(fn="any", values=np.array([5.0, 7.0]), background=0.0), np.full((1, 4, 4), 1.0)),
        # test-boundary.R:124-133 (by groups a, b)
        ("by_groups", halves, GRID4,
         dict(fn="last", values=np.array([10.0, 20.0]), background=0.0, bands=np.array([0, 1]), n_bands=2),
         np.stack([_m([[10, 10, 0, 0]] * 4), _m([[0, 0, 20, 20]] * 4)])),
        # test-geometry.R:9-15 (point (1.5, 1.5) -> row 2, col 1)
        ("point_cell", table(point(1.5, 1.5)), GRID4, dict(fn="last", values=9.0, background=0.0),
         _m([[0, 0, 0, 0], [0, 0, 0, 0], [0, 9, 0, 0], [0, 0, 0, 0]])[None]),
        # test-geometry.R:17-23 (diagonal line (0,0)-(4,4): 3 cells)
        ("diagonal_line", table(line([(0, 0), (4, 4)])), GRID4, dict(fn="last", values=9.0, background=0.0),
         _m([[0, 0, 0, 0], [0, 0, 0, 9], [0, 0, 9, 0], [0, 9, 0, 0]])[None]),
        # test-geometry.R:32-39 (multipolygon quadrants)
        ("multipolygon", table(mpoly(sq(0, 0, 2, 2), sq(2, 2, 4, 4))), GRID4,
         dict(fn="last", values=9.0, background=0.0),
         _m([[0, 0, 9, 9], [0, 0, 9, 9], [9, 9, 0, 0], [9, 9, 0, 0]])[None]),
        # test-geometry.R:41-46 (background -1)
        ("background_minus1", table(poly(sq(0, 0, 2, 2))), GRID4, dict(fn="last", values=9.0, background=-1.0),
         _m([[-1, -1, -1, -1], [-1, -1, -1, -1], [9, 9, -1, -1], [9, 9, -1, -1]])[None]),
        # test-geometry.R:48-51 (NA background, full coverage)
        ("background_nan", full, GRID4, dict(fn="last", values=3.0, background=np.nan), np.full((1, 4, 4), 3.0)),
    ]
    return kats


def rust_kats():
    """burn_geometry.rs tests (a 'last' raster of value 1 shows the written cells)."""
    def cells(rows_cols, grid=GRID10):
        m = np.zeros((1, grid["nrows"], grid["ncols"]))
        for r, c in rows_cols:
            m[0, r, c] = 1.0
        return m

    return [
        ("rust_point_exact_cell", table(point(2.5, 7.5)), GRID10, dict(fn="last", values=1.0, background=0.0),
         cells([(2, 2)])),
        ("rust_multipoint", table(mpoint([(1.5, 8.5), (5.5, 3.5)])), GRID10,
         dict(fn="last", values=1.0, background=0.0), cells([(1, 1), (6, 5)])),
        ("rust_horizontal_line", table(line([(1.0, 5.0), (6.0, 5.0)])), GRID10,
         dict(fn="last", values=1.0, background=0.0), lambda r: r[0].any() and (r[0].nonzero()[0] == 5).all()),
        ("rust_multilinestring", table(mline([[(1.0, 8.0), (4.0, 8.0)], [(1.0, 2.0), (4.0, 2.0)]])), GRID10,
         dict(fn="last", values=1.0, background=0.0), lambda r: r[0, 2].any() and r[0, 8].any()),
        ("rust_polygon_fills", table(poly(sq(2, 2, 6, 6))), GRID10, dict(fn="last", values=1.0, background=0.0),
         lambda r: (r > 0).sum() > 4),
        ("rust_collection", table(lambda b: (b.add_part(G.POINT, [(np.array([[2.5, 7.5]]), 0)]),
                                             b.add_part(G.POLYGON, [(np.array(sq(5, 1, 8, 4), float), 0)]),
                                             b.end_geometry())),
         GRID10, dict(fn="last", values=1.0, background=0.0),
         lambda r: r[0, 2, 2] == 1.0 and r[0, 6:].any()),
        # rasterize.rs:251-274
        ("rust_dense_polygon", table(poly([(0.5, 0.5), (3.5, 0.5), (3.5, 3.5), (0.5, 3.5), (0.5, 0.5)])), GRID4,
         dict(fn="last", values=1.0, background=0.0), lambda r: (r == 1.0).any()),
    ]


def all_kats():
    return r_kats() + rust_kats()
