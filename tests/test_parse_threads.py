"""WKT / WKB ingestion on several host threads (rz_parse_wkt / rz_parse_wkb
parse contiguous chunks of items in parallel and append the chunk tables):
the table, the dropped items and the reported error are those of a
sequential parse.  RZ_PARSE_THREADS forces the thread count.  CPU only."""

import os
import struct

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G

FIELDS = ("part_offsets", "part_kind", "ring_offsets", "vertex_offsets", "ring_flags", "xy")


def _with_threads(n, f, *a):
    old = os.environ.get("RZ_PARSE_THREADS")
    os.environ["RZ_PARSE_THREADS"] = str(n)
    try:
        return f(*a)
    finally:
        if old is None:
            del os.environ["RZ_PARSE_THREADS"]
        else:
            os.environ["RZ_PARSE_THREADS"] = old


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(getattr(a, f), getattr(b, f), equal_nan=True), f


def _wkt_items(rng, n):
    out = []
    for i in range(n):
        k = i % 6
        x, y = (float(v) for v in rng.uniform(-1e3, 1e3, 2))
        if k == 0:
            out.append(f"POINT ({x!r} {y!r})")
        elif k == 1:
            pts = ", ".join(f"{x + j!r} {y - j * 0.5!r}" for j in range(int(rng.integers(2, 9))))
            out.append(f"LINESTRING ({pts})")
        elif k == 2:
            out.append(f"POLYGON (({x} {y}, {x + 3} {y}, {x + 3} {y + 2}, {x} {y}), "
                       f"({x + 1} {y + 0.5}, {x + 2} {y + 0.5}, {x + 2} {y + 1}, {x + 1} {y + 0.5}))")
        elif k == 3:
            out.append(f"MULTIPOLYGON ((({x} {y}, {x + 1} {y}, {x + 1} {y + 1}, {x} {y})), "
                       f"(({x + 5} {y}, {x + 6} {y}, {x + 6} {y + 1}, {x + 5} {y})))")
        elif k == 4:
            out.append(f"GEOMETRYCOLLECTION (POINT ({x} {y}), LINESTRING ({x} {y}, {x + 2} {y + 2}))")
        else:
            out.append(f"MULTILINESTRING Z (({x} {y} 1, {x + 1} {y} 2), ({x} {y + 1} 3, {x + 2} {y + 3} 4))")
    return out


def test_wkt_parallel_parse_equals_sequential():
    items = _wkt_items(np.random.default_rng(5), 3001)
    seq = _with_threads(1, G.from_wkt, items)
    for t in (2, 7, 32):
        _same(_with_threads(t, G.from_wkt, items), seq)
    assert seq.n_geoms == 3001


def _wkb_point(x, y):
    return struct.pack("<BI", 1, 1) + struct.pack("<dd", x, y)


def test_wkb_parallel_parse_drops_empty_points_in_order():
    rng = np.random.default_rng(9)
    blobs = []
    for i in range(2000):
        if i % 7 == 3:
            blobs.append(_wkb_point(np.nan, np.nan))  # POINT EMPTY: dropped
        else:
            blobs.append(_wkb_point(*rng.uniform(-10, 10, 2)))
    seq = _with_threads(1, G.from_wkb, blobs)
    assert seq.n_geoms == 2000 - sum(1 for i in range(2000) if i % 7 == 3)
    for t in (3, 16):
        _same(_with_threads(t, G.from_wkb, blobs), seq)


@pytest.mark.parametrize("threads", [1, 4, 9])
def test_first_failing_item_is_reported(threads):
    items = _wkt_items(np.random.default_rng(1), 900)
    items[700] = "POLYGON ((0 0, 1 0"        # truncated
    items[123] = "LINESTRING (0 0, 1 x)"     # bad number: the first failure in item order
    with pytest.raises(rz.PanicException, match=r"WKT is valid\. \(item 123"):
        _with_threads(threads, G.from_wkt, items)
    blobs = [_wkb_point(1.0, 2.0)] * 500
    blobs[450] = b"\x01\x03\x00"
    blobs[77] = b"\x01\x02"
    with pytest.raises(rz.PanicException, match=r"WKB bytes are valid\. \(item 77"):
        _with_threads(threads, G.from_wkb, blobs)


def test_all_items_dropped_across_chunks():
    blobs = [_wkb_point(np.nan, np.nan)] * 300
    with pytest.raises(ValueError, match="Could not parse geometry"):
        _with_threads(6, G.from_wkb, blobs)
