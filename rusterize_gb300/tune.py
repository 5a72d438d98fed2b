"""Autotuner of the engine's schedule (``rz_tuning``).

The kernels have launch shapes and thresholds that change only their speed,
never a result (``include/rusterize_gb300.h``, rz_tuning): how many polygon
windows a warp takes per work grab, the grids of the span, scatter and line
kernels, the polygon window height, the width that separates the narrow
(warp per window) and wide (block per window) span kernels, and how many
records of a tile the fill sorts in one warp before it falls back to the
per-word path.  The best setting depends on the workload -- raster sides,
polygons per job and their size, the depth of overlap -- and on the device.

``autotune`` runs a workload callable under candidate settings on one GPU,
reads the device time the engine measured with CUDA events on its stream,
and keeps the fastest: a coordinate descent over the knobs, starting from
the defaults, a few rounds, the median of a few runs per candidate.  The
choice is cached per device and workload class in a JSON file
(``RUSTERIZE_GB300_TUNING``, else ``~/.cache/rusterize_gb300/tuning.json``),
so a long-running process tunes a class once.
"""

from __future__ import annotations

import json
import math
import os
import statistics
import threading
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable

# candidate values per knob; narrow_blocks_per_sm is bounded by the device's
# occupancy limit at run time
SPACE: dict[str, list[int]] = {
    "narrow_chunk": [1, 2, 4, 8, 16],
    "narrow_blocks_per_sm": [],  # filled from the context: limit, limit - 1, limit - 2
    "rows_per_window": [32, 64, 128],
    "narrow_max_words": [8, 16, 32],
    "fill_sort_max": [64, 128, 256],
    "scatter_blocks_per_sm": [4, 8, 16],
    "line_blocks_per_sm": [4, 8, 16],
}


@dataclass
class TuneResult:
    tuning: dict
    ms: float
    default_ms: float
    trials: list = field(default_factory=list)  # (tuning, ms) in the order tried

    def as_dict(self) -> dict:
        return {"tuning": self.tuning, "ms": self.ms, "default_ms": self.default_ms,
                "speedup": self.default_ms / self.ms if self.ms > 0 else None, "trials": len(self.trials)}


def _space_for(ctx) -> dict[str, list[int]]:
    space = {k: list(v) for k, v in SPACE.items()}
    limit = int(ctx.tuning["narrow_blocks_per_sm"]) if ctx is not None else 6
    space["narrow_blocks_per_sm"] = sorted({max(1, limit - 2), max(1, limit - 1), limit})
    return space


def coordinate_descent(measure: Callable[[dict], float], space: dict[str, list[int]], start: dict,
                       rounds: int = 2) -> TuneResult:
    """Minimise measure(setting) one knob at a time, `rounds` passes over the
    knobs, each knob tried at every candidate with the others fixed."""
    cache: dict[tuple, float] = {}
    trials: list = []

    def cost(setting: dict) -> float:
        key = tuple(sorted(setting.items()))
        if key not in cache:
            cache[key] = measure(dict(setting))
            trials.append((dict(setting), cache[key]))
        return cache[key]

    best = dict(start)
    best_ms = cost(best)
    default_ms = best_ms
    for _ in range(rounds):
        improved = False
        for knob, values in space.items():
            for v in values:
                if best.get(knob) == v:
                    continue
                cand = dict(best)
                cand[knob] = v
                ms = cost(cand)
                if ms < best_ms:
                    best, best_ms, improved = cand, ms, True
        if not improved:
            break
    return TuneResult(best, best_ms, default_ms, trials)


def autotune(ctx, run: Callable[[], float], *, rounds: int = 2, repeats: int = 3, warmup: int = 1,
             space: dict[str, list[int]] | None = None) -> TuneResult:
    """Tune `ctx` for the workload `run` (a callable that burns it once on
    `ctx` and returns the engine-measured device milliseconds).  The best
    setting is left on the context."""
    space = space or _space_for(ctx)
    start = ctx.tuning  # the defaults in force

    def measure(setting: dict) -> float:
        ctx.set_tuning(setting)
        for _ in range(warmup):
            run()
        return statistics.median(run() for _ in range(repeats))

    try:
        res = coordinate_descent(measure, space, start, rounds=rounds)
    finally:
        ctx.set_tuning(None)
    ctx.set_tuning(res.tuning)
    return res


# ---- workload classes and the cache -------------------------------------

def _log2_bin(x: float) -> int:
    return int(math.floor(math.log2(x))) if x >= 1 else 0


def batch_class(n_jobs: int, raster_px: float, n_geoms: float, n_vertices: float) -> str:
    """A class of batch workloads: power-of-two bins of the jobs, the mean
    raster pixels per job, polygons per job and vertices per polygon."""
    n = max(1, n_jobs)
    return (f"batch:jobs=2^{_log2_bin(n)}:px=2^{_log2_bin(raster_px / n)}:geoms=2^{_log2_bin(n_geoms / n)}"
            f":verts=2^{_log2_bin(n_vertices / max(1.0, n_geoms))}")


def table_class(nrows: int, ncols: int, n_geoms: int, n_vertices: int) -> str:
    """A class of single burns: power-of-two bins of the raster pixels,
    geometries and vertices per geometry."""
    return (f"single:px=2^{_log2_bin(float(nrows) * ncols)}:geoms=2^{_log2_bin(n_geoms)}"
            f":verts=2^{_log2_bin(n_vertices / max(1, n_geoms))}")


_cache_lock = threading.Lock()


def cache_path() -> Path:
    env = os.environ.get("RUSTERIZE_GB300_TUNING")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "rusterize_gb300" / "tuning.json"


def _read(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def cached(device_name: str, cls: str, path: Path | None = None) -> dict | None:
    """The cached tuning of (device, class), or None."""
    with _cache_lock:
        return _read(path or cache_path()).get(device_name, {}).get(cls, {}).get("tuning")


def store(device_name: str, cls: str, result: TuneResult, path: Path | None = None) -> None:
    path = path or cache_path()
    with _cache_lock:
        data = _read(path)
        data.setdefault(device_name, {})[cls] = result.as_dict()
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(path)


def tuned(ctx, device_name: str, cls: str, run: Callable[[], float], *, path: Path | None = None,
          **kw) -> tuple[dict, TuneResult | None]:
    """Apply the cached tuning of (device, class) to `ctx`, or tune it with
    `run` and cache the result.  Returns (tuning, result or None if cached)."""
    t = cached(device_name, cls, path)
    if t is not None:
        ctx.set_tuning(t)
        return t, None
    res = autotune(ctx, run, **kw)
    store(device_name, cls, res, path)
    return res.tuning, res
