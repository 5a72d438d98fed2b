"""The autotuner: its search on a synthetic cost (CPU), its cache and
workload classes (CPU), and on the GPU that every schedule gives
bit-identical rasters and that tuning a batch picks a valid setting."""

from __future__ import annotations

import numpy as np
import pytest

from rusterize_gb300 import tune


def test_coordinate_descent_finds_the_separable_optimum():
    space = {"a": [1, 2, 4, 8], "b": [10, 20, 30], "c": [0, 1]}
    best = {"a": 4, "b": 20, "c": 1}
    calls = []

    def measure(s):
        calls.append(s)
        return sum((np.log2(s[k] + 1) - np.log2(best[k] + 1)) ** 2 for k in s) + 1.0

    res = tune.coordinate_descent(measure, space, {"a": 1, "b": 10, "c": 0}, rounds=3)
    assert res.tuning == best
    assert res.ms == 1.0 and res.default_ms > res.ms
    assert len(calls) == len({tuple(sorted(c.items())) for c in calls})  # each setting measured once


def test_classes_bin_by_powers_of_two():
    a = tune.batch_class(3000, 3000 * 1.0e7, 3000 * 600, 3000 * 600 * 130)
    b = tune.batch_class(3500, 3500 * 1.2e7, 3500 * 700, 3500 * 700 * 140)
    assert a == b == "batch:jobs=2^11:px=2^23:geoms=2^9:verts=2^7"
    assert tune.table_class(20000, 20000, 100_000, 31_974_386) == "single:px=2^28:geoms=2^16:verts=2^8"


def test_cache_round_trip(tmp_path):
    path = tmp_path / "t.json"
    assert tune.cached("GB300", "x", path) is None
    res = tune.TuneResult({"narrow_chunk": 8}, 1.5, 2.0, [({}, 2.0), ({"narrow_chunk": 8}, 1.5)])
    tune.store("GB300", "x", res, path)
    tune.store("GB300", "y", tune.TuneResult({"narrow_chunk": 2}, 1.0, 1.0), path)
    assert tune.cached("GB300", "x", path) == {"narrow_chunk": 8}
    assert tune.cached("GB300", "y", path) == {"narrow_chunk": 2}
    assert tune.cached("other", "x", path) is None


@pytest.mark.gpu
def test_every_schedule_gives_the_same_raster():
    import rusterize_gb300 as rz
    from rusterize_gb300 import _lib, synth

    ctx = _lib.Context(0)
    a, b = synth.mixed(seed=5, scale=0.002)
    w = synth.large_fill(seed=9, scale=0.02, fn="sum")
    cases = [(a.table, rz.raster_info(a.table, res=a.res, extent=a.extent), b.values, "max", "int32", 0),
             (w.table, rz.raster_info(w.table, res=w.res, extent=w.extent), w.values, "sum", "float64", np.nan)]
    settings = [None,
                {"narrow_chunk": 1, "rows_per_window": 8, "narrow_max_words": 1, "fill_sort_max": 64,
                 "scatter_blocks_per_sm": 1, "line_blocks_per_sm": 1, "narrow_blocks_per_sm": 1,
                 "wide_blocks_per_sm": 1},
                {"narrow_chunk": 64, "rows_per_window": 32, "narrow_max_words": 8, "fill_sort_max": 128,
                 "scatter_blocks_per_sm": 32, "line_blocks_per_sm": 32}]
    for table, info, vals, fn, dt, bg in cases:
        ref = None
        for s in settings:
            ctx.set_tuning(s)
            got = rz.rasterize_table(table, info, values=vals, fn=fn, background=bg, dtype=dt, context=ctx)
            if ref is None:
                ref = got
            else:
                assert got.view(np.uint8).tobytes() == ref.view(np.uint8).tobytes(), s
    with pytest.raises(ValueError):
        ctx.set_tuning({"rows_per_window": 4})
    ctx.close()


@pytest.mark.gpu
def test_autotune_a_small_batch_picks_a_valid_setting(tmp_path):
    import rusterize_gb300 as rz
    from rusterize_gb300 import _lib, synth
    from rusterize_gb300.device import DeviceTable, rasterize_batch_device, upload
    from rusterize_gb300.engine import BatchJob

    ctx = _lib.Context(0)
    ws = synth.batch_jobs(seed=12, n_jobs=24, side_range=(256.0, 1024.0))
    jobs = [BatchJob(DeviceTable.upload(w.table), rz.raster_info(w.table, res=w.res, extent=w.extent),
                     upload(w.values), w.fn, w.background) for w in ws]
    outs = None

    def run():
        nonlocal outs
        st = {}
        outs = rasterize_batch_device(jobs, dtype="float32", outs=outs, context=ctx, stats=st)
        return st["ms_device_total"]

    res = tune.autotune(ctx, run, rounds=1, repeats=1, warmup=0,
                        space={"narrow_chunk": [1, 8], "fill_sort_max": [64, 256]})
    assert res.trials and res.ms <= res.default_ms
    assert ctx.tuning["narrow_chunk"] == res.tuning["narrow_chunk"]
    # the tuned schedule burns the same rasters
    before = [o.clone() for o in outs]
    ctx.set_tuning(None)
    run()
    assert all(bool((x == y).all()) for x, y in zip(before, outs))
    ctx.close()
