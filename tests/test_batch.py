"""rz_rasterize_batch: many independent jobs in one pass of the engine.

Every job's raster must be bit-identical to the one rz_rasterize returns
for that job alone (and so to the oracle's).  The jobs mix polygons with
holes, lines and points, every pixel function, backgrounds that put jobs in
different fill variants, square and non-square pixels, scalar / absent /
per-geometry values, empty jobs, and waves split by a small byte budget."""

import zlib

import numpy as np
import pytest

import rusterize_gb300 as rz
from rusterize_gb300 import geometry as G
from rusterize_gb300 import synth
from rusterize_gb300.engine import BatchJob, RasterInfo, rasterize_batch, rasterize_table

from _util import diff_report, oracle_burn, same_bits

pytestmark = pytest.mark.gpu

FNS = ["sum", "first", "last", "min", "max", "count", "any"]


def _job(rng, i, dtype):
    """A random job: its own extent, resolution, geometry mix, function,
    background and values."""
    kind = i % 5
    side = int(rng.integers(20, 700))
    res = (1.0, 1.0) if kind != 3 else (float(rng.uniform(0.4, 2.0)), float(rng.uniform(0.4, 2.0)))
    x0, y0 = float(rng.uniform(-1e4, 1e4)), float(rng.uniform(-1e4, 1e4))
    ncols, nrows = side, int(rng.integers(10, 700))
    info = RasterInfo(nrows=nrows, ncols=ncols, xmin=x0, xmax=x0 + ncols * res[0], ymin=y0,
                      ymax=y0 + nrows * res[1], xres=res[0], yres=res[1])
    w, h = ncols * res[0], nrows * res[1]
    parts = []
    n = int(rng.integers(0, 60)) if kind != 4 else 0
    if n:
        r = rng.uniform(1.0, 0.3 * max(w, h), n)
        parts.append(synth.star_polygons(rng, n, (3, 40), r, x0 + rng.uniform(-0.1 * w, 1.1 * w, n),
                                         y0 + rng.uniform(-0.1 * h, 1.1 * h, n), n_holes=rng.integers(0, 3, n)))
    if kind in (1, 2, 3):
        parts.append(synth.random_walk_lines(rng, int(rng.integers(1, 30)), (2, 20), (0.3, 0.2 * max(w, h)),
                                             (x0 - 5, y0 - 5, x0 + w + 5, y0 + h + 5)))
        parts.append(synth.random_points(rng, int(rng.integers(1, 40)), (x0, y0, x0 + w, y0 + h)))
    if parts:
        table = G.GeometryTable.concat(parts)
    else:
        table = G.TableBuilder().build()
    fn = FNS[int(rng.integers(0, len(FNS)))]
    bg = [0, 3, np.nan][i % 3] if np.dtype(dtype).kind == "f" else [0, 3, 7][i % 3]
    vkind = i % 4
    if vkind == 0:
        values = None
    elif vkind == 1:
        values = np.array(5, dtype=dtype)[()]
    else:
        values = rng.integers(1, 9, table.n_geoms).astype(dtype)
    return BatchJob(table=table, info=info, values=values, fn=fn, background=bg)


def _jobs(seed, n, dtype):
    rng = np.random.default_rng(seed)
    return [_job(rng, i, dtype) for i in range(n)]


def _single(job, dtype, all_touched=False):
    return rasterize_table(job.table, job.info, values=job.values, fn=job.fn, background=job.background, dtype=dtype,
                           all_touched=all_touched)


@pytest.mark.parametrize("dtype", ["float64", "float32", "uint16", "int32"])
def test_batch_equals_single_calls(dtype):
    jobs = _jobs(zlib.crc32(dtype.encode()), 60, dtype)
    st = {}
    outs = rasterize_batch(jobs, dtype=dtype, stats=st)
    assert st["jobs"] == 60 and st["waves"] == 1
    for i, (job, got) in enumerate(zip(jobs, outs)):
        want = _single(job, dtype)
        assert same_bits(got, want), f"job {i} ({job.fn}): " + diff_report(got, want)


def test_batch_matches_the_oracle():
    jobs = _jobs(5, 25, "float64")
    outs = rasterize_batch(jobs, dtype="float64")
    for i, (job, got) in enumerate(zip(jobs, outs)):
        vals = job.values
        ref = oracle_burn(job.table, job.info, fn=job.fn, values=vals, background=job.background, dtype="float64")
        assert same_bits(got, ref), f"job {i} ({job.fn}): " + diff_report(got, ref)


def test_batch_waves_and_all_touched():
    jobs = _jobs(17, 40, "float32")
    st = {}
    outs = rasterize_batch(jobs, dtype="float32", wave_bytes=1 << 20, stats=st)
    assert st["waves"] > 3
    for i, (job, got) in enumerate(zip(jobs, outs)):
        want = _single(job, "float32")
        assert same_bits(got, want), f"job {i}: " + diff_report(got, want)
    outs = rasterize_batch(jobs, dtype="float32", all_touched=True)
    for i, (job, got) in enumerate(zip(jobs, outs)):
        want = _single(job, "float32", all_touched=True)
        assert same_bits(got, want), f"job {i} all_touched: " + diff_report(got, want)


def test_batch_of_uneven_jobs_from_the_generator():
    # jobs of the uneven-size generator, reduced sides
    ws = synth.batch_jobs(seed=1004, n_jobs=24, side_range=(64.0, 1500.0), max_polygons=3000)
    jobs = [BatchJob(w.table, rz.raster_info(w.table, res=w.res, extent=w.extent), w.values, w.fn, w.background)
            for w in ws]
    outs = rasterize_batch(jobs, dtype="float32")
    for i, (job, got) in enumerate(zip(jobs, outs)):
        want = _single(job, "float32")
        assert same_bits(got, want), f"job {i}: " + diff_report(got, want)


def test_batch_device_inputs_and_outputs():
    torch = pytest.importorskip("torch")
    from rusterize_gb300.device import DeviceTable, rasterize_batch_device, upload

    jobs = _jobs(23, 30, "float64")
    djobs = []
    for j in jobs:
        v = j.values
        if isinstance(v, np.ndarray) and v.ndim == 1:
            v = upload(v)
        djobs.append(BatchJob(DeviceTable.upload(j.table), j.info, v, j.fn, j.background))
    outs = rasterize_batch_device(djobs, dtype="float64")
    for i, (job, got) in enumerate(zip(jobs, outs)):
        want = _single(job, "float64")
        g = got.cpu().numpy().view(np.float64).reshape(want.shape)
        assert same_bits(g, want), f"job {i}: " + diff_report(g, want)


def test_batch_rejects_an_inconsistent_device_table():
    torch = pytest.importorskip("torch")
    from rusterize_gb300.device import DeviceTable, rasterize_batch_device

    jobs = _jobs(29, 4, "float64")
    djobs = [BatchJob(DeviceTable.upload(j.table), j.info, None, j.fn, j.background) for j in jobs]
    bad = next(i for i, j in enumerate(djobs) if j.table.table.n_geoms > 0)
    djobs[bad].table.tensors["part_offsets"][-1] += 1  # last offset no longer equals n_parts
    with pytest.raises(ValueError, match=f"job {bad}"):
        rasterize_batch_device(djobs, dtype="float64")


def test_batch_argument_errors():
    jobs = _jobs(31, 3, "float64")
    jobs[1].fn = "median"
    with pytest.raises(ValueError, match="Unknown pixel function"):
        rasterize_batch(jobs, dtype="float64")
    assert rasterize_batch([], dtype="float64") == []
