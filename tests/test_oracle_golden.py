"""The oracle (CPU restatement) against the reference's own golden rasters
and known-answer tests.  CPU only."""

import numpy as np
import pytest

import oracle
from rusterize_gb300 import geometry as G

from _kats import all_kats
from _util import GOLDEN, explode, golden_inputs, oracle_burn


def test_golden_standard_output_sum():
    # python/test/test_many.py:228-235: rusterize(GDF, res=(1, 1), dtype="uint8", field="value", fun="sum")
    geoms, values = golden_inputs()
    t = G.from_wkt(geoms)
    info = oracle.raster_info(t, res=(1, 1))
    assert info[:2] == (131, 361)
    r = oracle_burn(t, info, fn="sum", values=values, background=0, dtype="uint8")
    gold = np.load(GOLDEN / "standard_output_sum.npy")
    assert np.array_equal(r[0], gold)


def test_golden_custom_shape():
    # python/test/test_many.py:329-346: exploded GDF, out_shape=(47, 319), fun="sum", uint8
    geoms, values = golden_inputs()
    t, v = explode(G.from_wkt(geoms), values)
    info = oracle.raster_info(t, shape=(47, 319))
    r = oracle_burn(t, info, fn="sum", values=v, background=0, dtype="uint8")
    gold = np.load(GOLDEN / "standard_output_sum_custom_shape.npy")
    assert np.array_equal(r[0], gold)


@pytest.mark.parametrize("kat", all_kats(), ids=lambda k: k[0])
def test_oracle_kats(kat):
    name, t, grid, kw, expected = kat
    r = oracle_burn(t, grid, **kw)
    if callable(expected):
        assert expected(r), name
    else:
        np.testing.assert_array_equal(r, expected)


def test_oracle_raster_info_kats():
    # test-boundary.R:97-106: shape-only (4,4) -> 4x4; resolution-only (1,1) -> 5x5 (half-pixel buffer)
    b = G.TableBuilder()
    G.add_polygon(b, [(0, 0), (4, 0), (4, 4), (0, 4)])
    t = b.build()
    assert oracle.raster_info(t, shape=(4, 4))[:2] == (4, 4)
    info = oracle.raster_info(t, res=(1, 1))
    assert info[:2] == (5, 5)
    assert info[2:6] == (-0.5, 4.5, -0.5, 4.5)
    with pytest.raises(ValueError, match="Unspecified extent"):
        oracle.raster_info(t, res=(1, 1), extent=(0, 0, 0, 0))
