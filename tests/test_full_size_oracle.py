"""Bit-exact parity against the oracle on the benchmark configurations at
their full sizes.

* Large fill: 100,000 star polygons with 0-3 holes over 20,000 x 20,000,
  `sum` into float64 (NaN background) and `count` into uint32 (background
  0), the two burns of one bench step.  The oracle runs each in about 4 s
  of one host thread.
* Mixed collection: 50,000 polygons + 200,000 linestrings + 1,000,000
  points over 40,000 x 40,000: the int32 `max` band of the category, and
  the 16 uint8 `any` bands of `by=str(category)`.  A `by` band is the burn
  of that group's geometries alone, in input order
  (rust/src/rasterize.rs:88-101, group_keys :198-205), so the oracle burns
  each band from its own geometries and the GPU band is compared with it.
* Uneven jobs: the first 64 jobs of the batched configuration (sides
  log-uniform up to 8,192, f32), each burned through the batched entry
  point and compared with the oracle; seven more jobs cover `any`.

Oracle calls run on host threads (ctypes releases the GIL), overlapping
the GPU burns.  Reference semantics: burners.rs:261-320 (polygon spans),
burners.rs:40-91 (lines), burners.rs:250-258 (points) and
pixel_functions.rs:56-122.
"""

from __future__ import annotations

import concurrent.futures as cf

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import synth

from _util import diff_report, oracle_burn, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _to_host(t) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_large_fill_full_size_sum_and_count_against_oracle():
    w = synth.large_fill(seed=1002, scale=1.0, fn="sum")
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    assert (info.nrows, info.ncols) == (20000, 20000) and w.table.n_geoms == 100_000
    with cf.ThreadPoolExecutor(2) as ex:
        f_sum = ex.submit(oracle_burn, w.table, info, fn="sum", values=w.values, background=np.nan,
                          dtype="float64")
        f_cnt = ex.submit(oracle_burn, w.table, info, fn="count", background=0, dtype="uint32")
        st: dict = {}
        got = rz.rasterize_table(w.table, info, values=w.values, fn="sum", background=np.nan, dtype="float64",
                                 stats=st)
        ref = f_sum.result()
        assert same_bits(got, ref), diff_report(got, ref)
        del got, ref
        got = rz.rasterize_table(w.table, info, fn="count", background=0, dtype="uint32")
        ref = f_cnt.result()
        assert same_bits(got, ref), diff_report(got, ref)
        assert int(got.sum(dtype=np.uint64)) == st["pixel_writes"]


def test_mixed_collection_full_size_max_and_any_bands_against_oracle():
    from rusterize_gb300.device import DeviceTable, rasterize_device, upload

    a, b = synth.mixed(seed=1003, scale=1.0)
    info = rz.raster_info(a.table, res=a.res, extent=a.extent)
    assert (info.nrows, info.ncols) == (40000, 40000)
    dt = DeviceTable.upload(a.table)
    with cf.ThreadPoolExecutor(8) as ex:
        f_max = ex.submit(oracle_burn, b.table, info, fn="max", values=b.values, background=0, dtype="int32")
        mx = rasterize_device(dt, info, fn="max", background=0, dtype="int32", values=upload(b.values))
        got = _to_host(mx)
        del mx
        ref = f_max.result()
        assert same_bits(got, ref), diff_report(got, ref)
        del got, ref

        bands = torch.from_numpy(a.bands.astype(np.int32)).cuda()
        anyr = rasterize_device(dt, info, fn="any", background=0, dtype="uint8", bands=bands, n_bands=a.n_bands)
        futs = {}
        for band in range(a.n_bands):
            sub = a.table.select(np.nonzero(a.bands == band)[0])
            futs[band] = ex.submit(oracle_burn, sub, info, fn="any", background=0, dtype="uint8")
        for band in range(a.n_bands):
            got = _to_host(anyr[band])
            ref = futs.pop(band).result()[0]
            assert same_bits(got, ref), f"band {band} ({a.meta['band_names'][band]}): " + diff_report(got, ref)


def test_uneven_jobs_full_size_against_oracle():
    from rusterize_gb300.engine import BatchJob, rasterize_batch

    ws = synth.batch_jobs(seed=1004, n_jobs=64)
    assert {w.fn for w in ws} == set(synth.BATCH_FNS)
    assert max(max(w.extent[2], w.extent[3]) for w in ws) > 4096
    jobs = []
    for w in ws:
        info = rz.raster_info(w.table, res=w.res, extent=w.extent)
        jobs.append(BatchJob(w.table, info, w.values, w.fn, w.background))
    # `any` and integer outputs are not drawn by the generator: cover them on seven more jobs
    extra = [BatchJob(j.table, j.info, None, "any", 0) for j in jobs[:7]]
    with cf.ThreadPoolExecutor(8) as ex:
        refs = [ex.submit(oracle_burn, j.table, j.info, fn=j.fn, values=j.values, background=j.background,
                          dtype="float32") for j in jobs]
        refs_any = [ex.submit(oracle_burn, j.table, j.info, fn="any", background=0, dtype="uint8") for j in extra]
        outs = rasterize_batch(jobs, dtype="float32")
        outs_any = rasterize_batch(extra, dtype="uint8")
        for i, (got, f) in enumerate(zip(outs, refs)):
            ref = f.result()
            assert same_bits(got, ref), f"job {i} ({jobs[i].fn}, {jobs[i].info.nrows}^2): " + diff_report(got, ref)
        for i, (got, f) in enumerate(zip(outs_any, refs_any)):
            ref = f.result()
            assert same_bits(got, ref), f"any job {i}: " + diff_report(got, ref)
    # the plain path on the same jobs: one call per job
    for i in (0, 1, 2, 3):
        j = jobs[i]
        got = rz.rasterize_table(j.table, j.info, values=j.values, fn=j.fn, background=j.background,
                                 dtype="float32")
        assert same_bits(got, outs[i])
