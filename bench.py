#!/usr/bin/env python
"""Benchmark of the plain burn path on the large polygon fill.

Workload (one "step"): 100,000 seeded star polygons with 0-3 holes (outer
ring 16-512 vertices, holes 8-64, radius lognormal median 20 px, max
2,000 px) over a 20,000 x 20,000 raster at resolution 1, burned twice on the
same inputs: pixel function 'sum' into float64 (NaN background) and 'count'
into uint32 (background 0).

  value : burned px/s (pixel writes per second) with inputs resident in HBM
          and rasters left on the device, CUDA events on the engine stream
  e2e   : the same metric through the public host API (rasterize_table) from
          pinned host buffers, H2D of the geometry and D2H of both rasters
          inside the timed region; the two burns are issued from two host
          threads on their own contexts, like the reference arm's two
          threads (the one-thread figure is reported beside it)
  cpu_baseline / --impl reference : the CPU restatement of the reference
          (oracle/), timed on this host on the same workload

Multi-GPU (torchrun, N > 1): by default every rank burns its own
independent job (seed + rank; "scaling": "weak"); with --shard rows every
rank burns its row band of the same job from the geometries that can write
there ("scaling": "strong").  No data-path collective either way.
"""

from __future__ import annotations

import argparse
import json
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "large_fill_100k_polygons_20000x20000_sum_f64+count_u32"
REF_THREADS = 2  # host threads of both CPU legs: one per burn of a step
REF_BUDGET_S = 100.0  # CPU seconds of timed steps in the reference arm (full-size steps, at least three)
METRIC = "burned px/s (large polygon fill: sum f64 + count u32)"


def _dist():
    from rusterize_gb300.shard import dist_env

    return dist_env()


def _workload(seed: int, scale: float):
    from rusterize_gb300 import synth

    w_sum = synth.large_fill(seed=seed, scale=scale, fn="sum")
    return w_sum


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        # the region starts once the sampler has written its first line
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            self.f.flush()
            if self.path.stat().st_size > 0:
                break
            time.sleep(0.02)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in self.path.read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 8:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx = float(parts[1])
                except ValueError:
                    continue
                for name, val in zip(names, parts[4:8]):
                    if val.lower() == "active":
                        reasons.add(name)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


class _nvtx:
    """An NVTX range around a leg, so that a profiler can select its launches."""

    def __init__(self, name: str):
        self.name = name

    def __enter__(self):
        import torch

        torch.cuda.nvtx.range_push(self.name)

    def __exit__(self, *a):
        import torch

        torch.cuda.nvtx.range_pop()


def _measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "fallback": True}


def _oracle_step(w_sum, info, threads: int = 2) -> tuple[float, int, int]:
    """One step of the CPU restatement: sum f64 and count u32 (independent
    calls, run in `threads` host threads).  Returns (seconds, px, edges)."""
    import oracle

    jobs = [("sum", "float64", w_sum.values, np.nan), ("count", "uint32", None, 0)]
    counters = [dict() for _ in jobs]

    def run(i):
        fn, dt, vals, bg = jobs[i]
        oracle.rasterize(w_sum.table, info.nrows, info.ncols, info.xmin, info.xmax, info.ymin, info.ymax, info.xres,
                         info.yres, values=vals, fn=fn, background=bg, dtype=dt, counters=counters[i])

    t0 = time.perf_counter()
    if threads > 1:
        ts = [threading.Thread(target=run, args=(i,)) for i in range(len(jobs))]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    else:
        for i in range(len(jobs)):
            run(i)
    dt_s = time.perf_counter() - t0
    return dt_s, sum(c["pixel_writes"] for c in counters), sum(c["edges"] for c in counters)


def run_reference(args) -> None:
    """The reference arm: the CPU restatement of the reference's burn path
    (oracle/) on this host, on the full workload of the GPU arm.  The two
    burns of a step (sum f64, count u32) run in REF_THREADS host threads, each
    single-threaded like the reference's single-band `process` loop
    (rust/src/rasterize.rs:105-113); the GPU arm's cpu_baseline uses the same
    threads."""
    rank, world, _ = _dist()
    if rank != 0:
        return
    import rusterize_gb300 as rz

    w = _workload(1002, args.scale)
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    # every step is the full workload (seconds of CPU each): the timed steps
    # stop at REF_BUDGET_S of CPU time, at least three, so that the arm ends
    # within a few minutes whatever --steps asks for
    warm = min(args.warmup, 2)
    for _ in range(warm):
        _oracle_step(w, info, threads=REF_THREADS)
    times, px, edges = [], 0, 0
    while len(times) < args.steps and (len(times) < 3 or sum(times) < REF_BUDGET_S):
        s, px, edges = _oracle_step(w, info, threads=REF_THREADS)
        times.append(s)
    ms = 1e3 * sum(times) / len(times)
    value = px / (ms / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "px/s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": warm, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "scale": args.scale, "polygons": w.table.n_geoms,
                   "vertices": w.table.n_vertices, "raster": [info.nrows, info.ncols]},
        "edges_per_s": edges / (ms / 1e3),
        "cpu_baseline": {"value": value, "unit": "px/s", "cores": REF_THREADS, "kind": "port",
                         "sample": f"the full workload every step ({w.table.n_geoms} polygons, {info.nrows} x "
                                   f"{info.ncols}): the two burns (sum f64, count u32) in {REF_THREADS} host threads, "
                                   "each single-threaded like the reference's single-band process loop"},
        "e2e": {"value": value, "unit": "px/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _roofline(ms, alg_step, nv, ng, acc, phase, hbm, args, peaks) -> dict:
    """Whole-step roofline (frac) and per-phase figures.

    frac = algorithmic bytes of the step / ms_per_step / measured HBM peak.
    Each phase is charged the algorithmic bytes it moves for the first time:
    the span kernels read the vertex table (16 B per vertex and call), the
    fill writes the rasters and reads the field values; prep re-reads the
    vertices (counted as traffic, not as algorithmic bytes) and the bucket
    phase only moves the engine's own coverage records."""
    out_bytes = acc[0][0]["out_bytes"] + acc[0][1]["out_bytes"]
    charged = {"ms_prep": 0, "ms_spans": 2 * 16 * nv, "ms_bucket": 0, "ms_fill": out_bytes + 8 * ng}
    kernels = {
        "ms_prep": "k_validate, k_part_geom, k_part_prep, scans, k_part_lists",
        "ms_spans": "k_poly_spans_narrow, k_poly_spans, k_line_spans, k_point_spans",
        "ms_bucket": "bucket scan, k_scatter",
        "ms_fill": "k_fill_warp, k_fill_big, k_fill_depth",
    }
    per_phase = {}
    for k, t in phase.items():
        gbs = charged[k] / (t / 1e3) / 1e9 if t > 0 else None
        per_phase[k[3:]] = {"kernels": kernels[k], "ms_per_step": t, "algorithmic_bytes": charged[k],
                            "gbs": gbs, "frac": gbs / hbm if gbs is not None else None}
    dom = max(per_phase, key=lambda k: per_phase[k]["ms_per_step"])
    achieved = alg_step / (ms / 1e3) / 1e9
    # DRAM bytes per step of every kernel from one-kernel ncu captures
    # (profiles/dram_traffic.json), when the workload matches
    traffic, traffic_src = None, None
    tpath = ROOT / "profiles" / "dram_traffic.json"
    if tpath.exists():
        t = json.loads(tpath.read_text())
        if t.get("workload") == WORKLOAD and float(t.get("scale", -1)) == float(args.scale):
            traffic = t.get("bytes_per_step")
            traffic_src = t.get("source")
    return {"bound": "hbm", "scope": "whole step (both calls)", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "target_frac": 0.60, "algorithmic_bytes_per_step": alg_step,
            "traffic": traffic, "traffic_source": traffic_src,
            "traffic_over_algorithmic": (traffic / alg_step) if traffic else None,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if not peaks.get("fallback") else "fallback",
            "dominant_phase": dom, "phases": per_phase,
            "records_per_step": acc[0][0]["spans"] + acc[0][1]["spans"]}


def run_gb300(args) -> None:
    import torch

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import rusterize_gb300 as rz
    from rusterize_gb300 import _lib
    from rusterize_gb300.device import DeviceTable, rasterize_device, upload

    ctx = _lib.Context(local)
    rows_split = args.shard == "rows" and world > 1
    # replicas: every rank burns its own job (seed + rank); rows: every rank
    # burns its row band of the same job, from the geometries that can write there
    w = _workload(1002 + (0 if rows_split else rank), args.scale)
    info = rz.raster_info(w.table, res=w.res, extent=w.extent)
    rows = None
    table, values = w.table, w.values
    if rows_split:
        from rusterize_gb300.shard import row_bands, select_rows

        rows = row_bands(info.nrows, world)[rank]
        idx = select_rows(w.table, info, *rows)
        table, values = w.table.select(idx), w.values[idx]
    nr = info.nrows if rows is None else rows[1] - rows[0]
    dtab = DeviceTable.upload(table, device=local)
    dvals = upload(values, device=local)
    out_sum = torch.empty((1, nr, info.ncols), dtype=torch.float64, device=f"cuda:{local}")
    out_cnt = torch.empty((1, nr, info.ncols), dtype=torch.int32, device=f"cuda:{local}")
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{local}")

    def step(stats_acc=None):
        st1, st2 = {}, {}
        rasterize_device(dtab, info, fn="sum", background=np.nan, dtype="float64", values=dvals, out=out_sum,
                         context=ctx, stats=st1, rows=rows)
        rasterize_device(dtab, info, fn="count", background=0, dtype="uint32", out=out_cnt, context=ctx, stats=st2,
                         rows=rows)
        if stats_acc is not None:
            stats_acc.append((st1, st2))
        return st1, st2

    from rusterize_gb300.shard import barrier, max_over_ranks, sum_over_ranks

    for _ in range(args.warmup):
        step()
    # the engine's schedule for this workload class, chosen by the autotuner
    # (outside the timed region; results do not depend on it)
    tuning = None
    if args.schedule:
        ctx.set_tuning(json.loads(args.schedule))
        tuning = {"tuning": ctx.tuning, "fixed": True}
    elif args.tune:
        from rusterize_gb300 import tune

        def step_ms():
            a, b = step()
            return a["ms_device_total"] + b["ms_device_total"]

        res = tune.autotune(ctx, step_ms, rounds=2, repeats=3, warmup=1)
        tuning = dict(res.as_dict(), workload_class=tune.table_class(info.nrows, info.ncols, table.n_geoms,
                                                                     table.n_vertices))
    acc: list = []
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk, _nvtx("large_fill"):
        ev0.record(stream)
        for _ in range(args.steps):
            step(acc)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    px_step = sum(s1["pixel_writes"] + s2["pixel_writes"] for s1, s2 in acc) / len(acc)
    edges_step = sum(s1["edges"] + s2["edges"] for s1, s2 in acc) / len(acc)
    launches = sum(s1["kernel_launches"] + s2["kernel_launches"] for s1, s2 in acc)
    phase = {k: float(np.mean([s1[k] + s2[k] for s1, s2 in acc]))
             for k in ("ms_prep", "ms_spans", "ms_bucket", "ms_fill")}
    # algorithmic bytes of one step (both calls), the per-job figure of the
    # measurement plan: 16 B per vertex (f64 x, y) + the field values read
    # + every output pixel written once (background included)
    nv, ng = table.n_vertices, table.n_geoms
    alg_sum = 16 * nv + 8 * ng + acc[0][0]["out_bytes"]
    alg_cnt = 16 * nv + acc[0][1]["out_bytes"]  # count burns T::one(): no field read
    alg_step = alg_sum + alg_cnt
    # the slowest rank's step time; the pixel writes of every rank (each burns
    # its own job: seed + rank)
    dev = torch.device("cuda", local)
    ms = max_over_ranks(ms, device=dev)
    px_all = sum_over_ranks(px_step, device=dev)
    edges_all = sum_over_ranks(edges_step, device=dev)
    value = px_all / (ms / 1e3)

    # e2e: public host API from pinned buffers (H2D + D2H inside the region)
    e2e = None
    if args.e2e:
        def pinned(a, fill=True):
            buf = torch.empty(max(1, a.nbytes), dtype=torch.uint8, pin_memory=True)
            arr = buf.numpy()[: a.nbytes].view(a.dtype).reshape(a.shape)
            if fill:
                arr[...] = a
            return arr

        tb = table
        ptab = rz.GeometryTable(pinned(tb.part_offsets), pinned(tb.part_kind), pinned(tb.ring_offsets),
                                pinned(tb.vertex_offsets), pinned(tb.ring_flags), pinned(tb.xy))
        pvals = pinned(values)
        o_sum = pinned(np.empty((1, nr, info.ncols), np.float64), fill=False)
        o_cnt = pinned(np.empty((1, nr, info.ncols), np.uint32), fill=False)

        e_stats: list = []
        # The two burns of a step as two independent calls, each on its own
        # engine context (stream), from two host threads -- the way the
        # reference arm runs them -- so that one call's host->device upload
        # and kernels overlap the other's device->host copy.  With
        # --e2e-threads 1 they run one after the other on one context.
        import concurrent.futures as cf

        ctx2 = _lib.Context(local) if args.e2e_threads > 1 else ctx
        pool = cf.ThreadPoolExecutor(2) if args.e2e_threads > 1 else None

        def burn_sum(st):
            rz.rasterize_table(ptab, info, values=pvals, fn="sum", background=np.nan, dtype="float64", out=o_sum,
                               context=ctx, stats=st, rows=rows)

        def burn_count(st):
            rz.rasterize_table(ptab, info, values=None, fn="count", background=0, dtype="uint32", out=o_cnt,
                               context=ctx2, stats=st, rows=rows)

        def host_step(keep=False, threads=args.e2e_threads):
            s1, s2 = {}, {}
            if threads > 1:
                f1, f2 = pool.submit(burn_sum, s1), pool.submit(burn_count, s2)
                f1.result()
                f2.result()
            else:
                burn_sum(s1)
                burn_count(s2)
            if keep:
                e_stats.append((s1, s2))

        def timed_steps(threads):
            host_step(threads=threads)
            barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e_stats.clear()
            e0.record(stream)
            for _ in range(args.e2e_steps):
                host_step(keep=True, threads=threads)
            e1.record(stream)
            torch.cuda.synchronize()
            return max_over_ranks(e0.elapsed_time(e1) / args.e2e_steps, device=dev)

        e_ms_seq = timed_steps(1) if args.e2e_threads > 1 else None
        e_ms = timed_steps(args.e2e_threads)
        if pool is not None:
            pool.shutdown()
        h2d = sum(a.nbytes for a in (tb.part_offsets, tb.part_kind, tb.ring_offsets, tb.vertex_offsets, tb.xy))
        h2d = 2 * h2d + values.nbytes
        d2h = o_sum.nbytes + o_cnt.nbytes
        # the engine's own events: host->device copies before the prep, and
        # the device->host tail after the last fill (copies that overlap the
        # fill are inside ms_fill)
        ms_h2d = float(np.mean([a["ms_h2d"] + b["ms_h2d"] for a, b in e_stats]))
        ms_d2h = float(np.mean([a["ms_d2h"] + b["ms_d2h"] for a, b in e_stats]))
        ms_dev = float(np.mean([a["ms_device_total"] + b["ms_device_total"] for a, b in e_stats]))
        e2e = {"value": px_all / (e_ms / 1e3), "unit": "px/s", "ms_per_step": e_ms,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_h2d_per_step": ms_h2d, "ms_d2h_tail_per_step": ms_d2h, "ms_engine_per_step": ms_dev,
               "h2d_gbs": h2d / (ms_h2d / 1e3) / 1e9 if ms_h2d > 0 else None,
               "host_link_gbs": (h2d + d2h) / (e_ms / 1e3) / 1e9,
               "buffers": "pinned host memory (torch pin_memory)",
               "host_threads": args.e2e_threads,
               "sequential_ms_per_step": e_ms_seq}

    peaks = _measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    roofline = _roofline(ms, alg_step, nv, ng, acc, phase, hbm, args, peaks)

    batched = _batched_leg(args, ctx, local) if (world == 1 and args.batch_jobs > 0) else None
    served = _served_leg(args, local) if (world == 1 and args.serve_seconds > 0) else None

    cpu = None
    if rank == 0 and world == 1 and args.cpu_baseline:
        s, cpx, _ = _oracle_step(w, info, threads=REF_THREADS)
        cpu = {"value": cpx / s, "unit": "px/s", "cores": REF_THREADS, "kind": "port",
               "sample": f"one step of the full workload (sum f64 + count u32) in {REF_THREADS} host threads, "
                         "one per burn, oracle/ restatement"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "px/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong" if rows_split else "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "scale": args.scale, "polygons": w.table.n_geoms,
                       "shard": ("row bands of one job" if rows_split else "one job per rank") if world > 1 else None,
                       "vertices": w.table.n_vertices, "raster": [info.nrows, info.ncols],
                       "l2": "inputs larger than L2 (vertex table and rasters exceed 129 MB); no flush"},
            "edges_per_s": edges_all / (ms / 1e3),
            "pixel_writes_per_step": px_step,
            "clocks": clk.summary(),
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": roofline,
            "tuning": tuning,
            "cpu_baseline": cpu,
            "batched": batched,
            "served": served,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def _batched_leg(args, ctx, local) -> dict:
    """Uneven independent jobs (synth.batch_jobs_fast: polygons per job
    lognormal median 500, sides log-uniform 256-8192, f32, pixel functions
    drawn per job; 4,096 jobs by default), device-resident: the plain path
    (one rz_rasterize per job) against the batched form (rz_rasterize_batch
    over all jobs), jobs/s and px/s, each with the schedule the autotuner
    picks for it on a sample of the jobs."""
    import torch

    import rusterize_gb300 as rz
    from rusterize_gb300 import synth
    from rusterize_gb300.device import DeviceTable, rasterize_batch_device, rasterize_device, upload
    from rusterize_gb300.engine import BatchJob

    ws = synth.batch_jobs_fast(seed=1004, n_jobs=args.batch_jobs)
    dev = torch.device("cuda", local)
    jobs, outs = [], []
    for w in ws:
        info = rz.raster_info(w.table, res=w.res, extent=w.extent)
        jobs.append(BatchJob(DeviceTable.upload(w.table, device=local), info, upload(w.values, device=local), w.fn,
                             w.background))
        outs.append(torch.empty(info.nrows * info.ncols * 4, dtype=torch.uint8, device=dev))
    px = sum(j.info.nrows * j.info.ncols for j in jobs)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def plain():
        for j, o in zip(jobs, outs):
            rasterize_device(j.table, j.info, fn=j.fn, background=j.background, dtype="float32", values=j.values,
                             out=o, context=ctx)

    st: dict = {}

    wave_bytes = int(args.batch_wave_gb * (1 << 30))

    def batch():
        rasterize_batch_device(jobs, dtype="float32", outs=outs, context=ctx, stats=st, wave_bytes=wave_bytes)

    def timed(f, reps):
        for _ in range(args.batch_warmup):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            f()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # each leg runs with its own schedule, tuned on a sample of the jobs
    from rusterize_gb300 import tune

    # the plain leg is tuned on a sample (one call per job is slow); the
    # batched leg, one call over all jobs in well under a second, on the
    # whole batch
    ns = min(len(jobs), max(1, args.batch_tune_jobs))
    sample_j, sample_o = jobs[:ns], outs[:ns]

    def plain_sample_ms():
        tot = 0.0
        for j, o in zip(sample_j, sample_o):
            st1: dict = {}
            rasterize_device(j.table, j.info, fn=j.fn, background=j.background, dtype="float32", values=j.values,
                             out=o, context=ctx, stats=st1)
            tot += st1["ms_device_total"]
        return tot

    def batch_ms():
        st1: dict = {}
        rasterize_batch_device(jobs, dtype="float32", outs=outs, context=ctx, stats=st1, wave_bytes=wave_bytes)
        return st1["ms_device_total"]

    legs = set(args.batch_legs.split(","))
    tunings = {}
    ms_plain = ms_batch = float("nan")
    if "plain" in legs:
        if args.tune:
            tunings["plain"] = tune.autotune(ctx, plain_sample_ms, rounds=1, repeats=1, warmup=1).as_dict()
        with _nvtx("batch_plain"):
            ms_plain = timed(plain, args.batch_steps)
    if "batched" in legs:
        if args.tune:
            ctx.set_tuning(None)
            tunings["batched"] = tune.autotune(ctx, batch_ms, rounds=2, repeats=2, warmup=1).as_dict()
        with _nvtx("batch_batched"):  # ncu --nvtx --nvtx-include "batch_batched/" selects these launches
            ms_batch = timed(batch, args.batch_steps)
    ctx.set_tuning(None)
    n = len(jobs)
    out = {
        "workload": f"uneven_jobs_{n}_sides_256-8192_f32",
        "jobs": n, "polygons": int(sum(j.table.table.n_geoms for j in jobs)), "raster_px": int(px),
        "plain": {"ms": ms_plain, "jobs_per_s": n / (ms_plain / 1e3), "px_per_s": px / (ms_plain / 1e3)},
        "batched": {"ms": ms_batch, "jobs_per_s": n / (ms_batch / 1e3), "px_per_s": px / (ms_batch / 1e3),
                    "waves": st.get("waves"), "kernel_launches": st.get("kernel_launches")},
        "batched_over_plain": ms_plain / ms_batch,
        "tuning": dict(tunings, sample_jobs={"plain": ns, "batched": n},
                       workload_class=tune.batch_class(n, px, sum(j.table.table.n_geoms for j in jobs),
                                                       sum(j.table.table.n_vertices for j in jobs))),
        "note": "device-resident geometry and rasters; CUDA events on the engine stream; outputs larger than L2",
    }
    del jobs, outs
    torch.cuda.empty_cache()
    return out


def _served_leg(args, local) -> dict:
    """A served stream: Poisson arrivals drawn from a pool of uneven jobs
    (sides log-uniform 256-16384, float32 and uint8 outputs) whose geometry
    is resident on the device, for `serve_seconds` per rate.  The batching
    server (two streams, `serve_budget_gb` admission budget) against the same
    server with one job per call on one stream (the plain path), at every
    rate up to `serve_plain_max_rate`.  Each result is released as soon as it
    completes.  px/s counts the raster pixels of the completed jobs."""
    import torch

    import rusterize_gb300 as rz
    from rusterize_gb300 import synth
    from rusterize_gb300.device import DeviceTable, upload
    from rusterize_gb300.engine import BatchJob
    from rusterize_gb300.serve import BurnServer

    ws = synth.batch_jobs(seed=1005, n_jobs=args.serve_pool, side_range=(256.0, 16384.0))
    pool = []
    for i, w in enumerate(ws):
        dtype = "float32" if i % 2 == 0 else "uint8"
        vals = w.values if dtype == "float32" else (1 + w.values * 254).astype(np.uint8)
        info = rz.raster_info(w.table, res=w.res, extent=w.extent)
        bg = w.background if dtype == "float32" else 0
        pool.append((BatchJob(DeviceTable.upload(w.table, device=local), info, upload(vals, device=local), w.fn, bg),
                     dtype))
    free, _ = torch.cuda.mem_get_info(local)
    budget = int(min(args.serve_budget_gb * (1 << 30), 0.5 * free))

    def run(rate, batched):
        rng = np.random.default_rng(int(rate) * 7 + batched)
        lat, errors, lock = [], [], threading.Lock()
        px_done = [0]
        done = threading.Event()
        n_sub = [0]

        def on_done(f):
            r = None
            try:
                r = f.result()
            except BaseException as e:  # a failed or cancelled request still ends
                with lock:
                    errors.append(repr(e)[:200])
            with lock:
                if r is not None:
                    lat.append(r.latency)
                    px_done[0] += f.px
                finished = len(lat) + len(errors) == n_sub[0] and closed[0]
            if r is not None:
                r.release()
            if finished:
                done.set()

        closed = [False]
        cancelled = [0]
        srv = BurnServer(device=local, budget_bytes=budget, streams=2 if batched else 1,
                         max_batch=args.serve_max_batch if batched else 1)
        try:
            t0 = time.perf_counter()
            t_next = t0
            while True:
                t_next += float(rng.exponential(1.0 / rate))
                if t_next - t0 > args.serve_seconds:
                    break
                delay = t_next - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                job, dtype = pool[int(rng.integers(0, len(pool)))]
                with lock:
                    n_sub[0] += 1
                fut = srv.submit(job, dtype=dtype)
                fut.px = job.info.nrows * job.info.ncols
                fut.add_done_callback(on_done)
            with lock:
                closed[0] = True
                if len(lat) + len(errors) == n_sub[0]:
                    done.set()
            # a saturated server's backlog is cut off after the drain limit:
            # what has not started by then is cancelled and reported
            if not done.wait(args.serve_drain_limit):
                cancelled[0] = srv.cancel_pending()
                done.wait(600)
            t_end = time.perf_counter()
            batches = srv.batches
            dev_ms, call_ms = srv.device_ms, srv.call_ms
        finally:
            srv.close()
        a = np.array(lat) * 1e3
        if len(errors) > cancelled[0]:
            print(f"served leg: {len(errors) - cancelled[0]} failed requests, first: {errors[0]}", file=sys.stderr)
        return {"submitted": n_sub[0], "completed": len(lat), "failed": len(errors) - cancelled[0],
                "jobs_per_s": len(lat) / (t_end - t0), "px_per_s": px_done[0] / (t_end - t0),
                "p50_ms": float(np.percentile(a, 50)) if len(a) else None,
                "p99_ms": float(np.percentile(a, 99)) if len(a) else None, "batches": batches,
                "drain_s": t_end - t0 - args.serve_seconds, "cancelled_after_drain_limit": cancelled[0],
                "device_ms": dev_ms, "batch_call_ms": call_ms,
                "device_busy": dev_ms / 1e3 / (t_end - t0) / (2 if batched else 1)}

    rates = []
    for rate in [float(r) for r in args.serve_rates.split(",") if r]:
        row = {"rate": rate, "batched": run(rate, True)}
        if rate <= args.serve_plain_max_rate:
            row["plain"] = run(rate, False)
        rates.append(row)
    del pool
    torch.cuda.empty_cache()
    return {"workload": f"served_pool_{len(ws)}_sides_256-16384_f32_u8", "seconds_per_rate": args.serve_seconds,
            "budget_bytes": budget, "max_batch": args.serve_max_batch, "rates": rates,
            "note": "Poisson arrivals; latency = completion - submission; throughput over arrival window + drain"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--shard", choices=["jobs", "rows"], default="jobs",
                    help="N > 1: independent jobs per rank (weak scaling) or row bands of one job (strong)")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-threads", type=int, default=2, choices=[1, 2],
                    help="host threads issuing the two burns of an e2e step (2: concurrent, own contexts)")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--batch-jobs", type=int, default=4096, help="jobs of the batched leg (0: skip it)")
    ap.add_argument("--batch-tune-jobs", type=int, default=512,
                    help="jobs of the sample the plain leg is tuned on (the batched leg is tuned on all jobs)")
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="run with the default schedule")
    ap.add_argument("--schedule", default=None,
                    help='fixed schedule of the large-fill leg instead of tuning, e.g. \'{"fill_sort_max": 128}\'')
    ap.add_argument("--batch-wave-gb", type=float, default=0.0,
                    help="byte budget of one wave of the batched call (0: the engine's default, 32 GiB)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--batch-warmup", type=int, default=1)
    ap.add_argument("--batch-legs", default="plain,batched", help="legs of the batched comparison to run")
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="arrival window per rate (0: skip)")
    ap.add_argument("--serve-rates", default="200,1000,5000")
    ap.add_argument("--serve-plain-max-rate", type=float, default=5000.0)
    ap.add_argument("--serve-pool", type=int, default=96)
    ap.add_argument("--serve-budget-gb", type=float, default=32.0)
    ap.add_argument("--serve-max-batch", type=int, default=512)
    ap.add_argument("--serve-drain-limit", type=float, default=10.0,
                    help="seconds to wait for the backlog after the arrival window before cancelling it")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
