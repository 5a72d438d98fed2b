"""Full-size checks on the large fill and the mixed collection, through
properties that hold at any size.  They add to the bit-exact oracle
comparisons of test_full_size_oracle.py: each identity pits two GPU paths
against each other (the ordered fill against the order-free one, write
order against value order).

Large fill (100,000 polygons, 20,000 x 20,000):
  * `sum` of ones (float64, background 0) equals `count` exactly: every sum
    of ones is an exact integer in f64.  The ordered fill and the order-free
    depth fill must agree.
  * `any` equals `count > 0`.
  * With the geometry index as the burn value, `first` equals `min` and
    `last` equals `max`.  Geometries burn in index order
    (rust/src/rasterize.rs:162-196), so the first writer of a pixel has its
    smallest index.
  * The sum of the `count` raster equals the pixel writes the call reports.
Mixed collection (50,000 polygons, 200,000 lines, 1,000,000 points,
40,000 x 40,000, 16 `by` bands):
  * The int32 `max` raster of the category equals, per pixel, the largest
    category among the 16 uint8 `any` bands that are set."""

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _burn(dt, info, **kw):
    from rusterize_gb300.device import rasterize_device

    return rasterize_device(dt, info, **kw)


def test_large_fill_full_size_identities():
    from rusterize_gb300.device import DeviceTable, upload

    w = synth.large_fill(seed=1002, scale=1.0, fn="sum")
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    dt = DeviceTable.upload(w.table)
    st = {}
    count = _burn(dt, info, fn="count", background=0, dtype="int32", stats=st)
    assert int(count.sum(dtype=torch.int64).item()) == st["pixel_writes"]
    ones = _burn(dt, info, fn="sum", background=0.0, dtype="float64", values=upload(np.ones(w.table.n_geoms)))
    assert torch.equal(ones, count.to(torch.float64))
    del ones
    anyr = _burn(dt, info, fn="any", background=0, dtype="uint8")
    assert torch.equal(anyr, (count > 0).to(torch.uint8))
    del anyr, count
    idx = upload(np.arange(w.table.n_geoms, dtype=np.float64))
    first = _burn(dt, info, fn="first", background=-1.0, dtype="float64", values=idx)
    mn = _burn(dt, info, fn="min", background=-1.0, dtype="float64", values=idx)
    assert torch.equal(first, mn)
    del first, mn
    last = _burn(dt, info, fn="last", background=-1.0, dtype="float64", values=idx)
    mx = _burn(dt, info, fn="max", background=-1.0, dtype="float64", values=idx)
    assert torch.equal(last, mx)


def test_mixed_collection_full_size_max_equals_any_bands():
    from rusterize_gb300.device import DeviceTable, upload

    a, b = synth.mixed(seed=1003, scale=1.0)
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    dt = DeviceTable.upload(a.table)
    bands = torch.from_numpy(a.bands.astype(np.int32)).cuda()
    anyr = _burn(dt, info, fn="any", background=0, dtype="uint8", bands=bands, n_bands=a.n_bands)
    mx = _burn(dt, info, fn="max", background=0, dtype="int32", values=upload(b.values))
    want = torch.zeros((info.nrows, info.ncols), dtype=torch.int32, device="cuda")
    for band, name in enumerate(a.meta["band_names"]):
        cat = int(name)
        want = torch.maximum(want, anyr[band].to(torch.int32) * cat)
    assert torch.equal(mx[0], want)
