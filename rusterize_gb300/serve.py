"""A burn server: continuous batching of independent burn requests.

Requests arrive at any time with device-resident geometry (a DeviceTable, as
uploaded once by the client) and are admitted against a device-memory
budget: an admitted request reserves the bytes of its raster, and requests
wait while the reservations would exceed the budget.  Each scheduler thread
owns one engine context (one CUDA stream).  It takes every admitted request
that has not started and has the same output type as the oldest one, and it
runs them as one `rz_rasterize_batch` call: one pass of the kernels for all
of them.  With two schedulers, requests that arrive while one batch is on
the GPU form the next batch on the other stream, so the two batches overlap
on the device.  A request's result is its raster in device memory, and it is
bit-identical to a single `rz_rasterize` of the same job.  The reservation
is returned when the client releases the result.

There is no counterpart in the reference, which burns one raster per call
(rust/src/rasterize.rs:54-116).
"""

from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .engine import BatchJob


@dataclass
class Request:
    job: BatchJob
    dtype: str
    nbytes: int
    future: Future
    t_submit: float
    t_start: float = 0.0
    t_done: float = 0.0


@dataclass
class Result:
    """A completed request: its raster (a CUDA tensor of raw bytes, nrows *
    ncols values of the request's dtype) and its timeline."""

    out: object
    t_submit: float
    t_start: float
    t_done: float
    batch_jobs: int
    _server: "BurnServer" = field(repr=False, default=None)
    _nbytes: int = 0
    _released: bool = False

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit

    def release(self) -> None:
        """Hand the raster's bytes back to the admission budget."""
        if not self._released and self._server is not None:
            self._released = True
            self.out = None
            self._server._release(self._nbytes)


class Admission:
    """The admission queue of a BurnServer, free of any GPU state.

    Requests wait in arrival order.  A batch is taken from the front: the
    requests of the oldest request's dtype, in arrival order, as long as
    their bytes fit the budget next to the bytes already reserved.  Its bytes
    stay reserved until `release`."""

    def __init__(self, budget_bytes: int, max_batch: int):
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)
        self._cv = threading.Condition()
        self._pending: collections.deque = collections.deque()
        self.reserved = 0
        self.peak_reserved = 0
        self.closing = False

    def put(self, req) -> None:
        if req.nbytes > self.budget:
            raise ValueError(f"request needs {req.nbytes} bytes, more than the server's budget of {self.budget}")
        with self._cv:
            if self.closing:
                raise RuntimeError("server is closed")
            self._pending.append(req)
            self._cv.notify()

    def take(self, timeout: float | None = None) -> list:
        """The next batch; [] once closed and drained (or on timeout)."""
        deadline = None if timeout is None else time.perf_counter() + timeout
        with self._cv:
            while True:
                if self._pending and self.reserved + self._pending[0].nbytes <= self.budget:
                    break
                if self.closing and not self._pending:
                    return []
                left = None if deadline is None else deadline - time.perf_counter()
                if left is not None and left <= 0:
                    return []
                self._cv.wait(left)
            dtype = self._pending[0].dtype
            # cost proportional to the requests looked at, not to the backlog: the skipped ones
            # go back to the front of the queue in their order
            batch, skipped = [], []
            while self._pending and len(batch) < self.max_batch:
                r = self._pending.popleft()
                if r.dtype == dtype and self.reserved + r.nbytes <= self.budget:
                    self.reserved += r.nbytes
                    batch.append(r)
                else:
                    skipped.append(r)
                    if r.dtype == dtype:  # arrival order within a dtype: nothing overtakes it
                        break
            self._pending.extendleft(reversed(skipped))
            self.peak_reserved = max(self.peak_reserved, self.reserved)
            return batch

    def release(self, nbytes: int) -> None:
        with self._cv:
            self.reserved -= nbytes
            self._cv.notify_all()

    def close(self) -> None:
        with self._cv:
            self.closing = True
            self._cv.notify_all()

    def cancel_pending(self) -> list:
        """Remove and return the requests that have not been taken yet."""
        with self._cv:
            out = list(self._pending)
            self._pending.clear()
            self._cv.notify_all()
            return out

    def __len__(self) -> int:
        with self._cv:
            return len(self._pending)


class BurnServer:
    """Continuous batching of burn requests on one GPU.

    budget_bytes: device bytes that admitted, unreleased rasters may hold.
    streams: scheduler threads, each with its own engine context.
    max_batch: most requests per batch call."""

    def __init__(self, *, device: int = 0, budget_bytes: int = 120 << 30, streams: int = 2, max_batch: int = 4096,
                 wave_bytes: int = 0):
        import torch

        self._torch = torch
        self.device = device
        self.wave_bytes = int(wave_bytes)
        self.admission = Admission(budget_bytes, max_batch)
        self._stats_lock = threading.Lock()
        self.batches = 0
        self.jobs_done = 0
        self.device_ms = 0.0  # engine-measured device time of every batch call, summed over streams
        self.call_ms = 0.0    # host time inside the batch calls (allocation + call), summed
        self._contexts = [_lib.Context(device) for _ in range(max(1, streams))]
        self._threads = [threading.Thread(target=self._run, args=(c,), daemon=True) for c in self._contexts]
        for t in self._threads:
            t.start()

    # ---- client side ----
    def submit(self, job: BatchJob, dtype: str = "float32") -> Future:
        """Queue one request; the future resolves to a Result."""
        if dtype not in _lib.DTYPES:
            raise ValueError(f"Unsupported dtype {dtype!r}")
        nbytes = int(job.info.nrows) * int(job.info.ncols) * np.dtype(dtype).itemsize
        fut: Future = Future()
        self.admission.put(Request(job, dtype, nbytes, fut, time.perf_counter()))
        return fut

    def cancel_pending(self) -> int:
        """Fail every request that has not started (its future raises
        CancelledError); running batches finish.  Returns how many."""
        from concurrent.futures import CancelledError

        reqs = self.admission.cancel_pending()
        for r in reqs:
            r.future.set_exception(CancelledError("request cancelled before it started"))
        return len(reqs)

    def close(self) -> None:
        """Finish the queued requests and stop the schedulers."""
        self.admission.close()
        for t in self._threads:
            t.join()
        for c in self._contexts:
            c.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- schedulers ----
    def _release(self, nbytes: int) -> None:
        self.admission.release(nbytes)

    def _run(self, ctx: _lib.Context) -> None:
        from .device import rasterize_batch_device

        torch = self._torch
        dev = torch.device("cuda", self.device)
        torch.cuda.set_device(dev)
        while True:
            batch = self.admission.take()
            if not batch:
                return
            t0 = time.perf_counter()
            outs = None
            try:
                outs = [torch.empty(max(1, r.nbytes), dtype=torch.uint8, device=dev) for r in batch]
                torch.cuda.current_stream(dev).synchronize()  # allocations ordered before the engine stream
                st: dict = {}
                rasterize_batch_device([r.job for r in batch], dtype=batch[0].dtype, outs=outs, context=ctx,
                                       wave_bytes=self.wave_bytes, stats=st)
            except Exception as e:  # every request of the batch sees the error; later batches go on
                outs = None
                for r in batch:
                    self._release(r.nbytes)
                    r.future.set_exception(e)
                continue
            t1 = time.perf_counter()
            with self._stats_lock:
                self.batches += 1
                self.jobs_done += len(batch)
                self.device_ms += float(st.get("ms_device_total", 0.0))
                self.call_ms += (t1 - t0) * 1e3
            results = [Result(o, r.t_submit, t0, t1, len(batch), self, r.nbytes) for r, o in zip(batch, outs)]
            del outs  # the results own the rasters now: a release frees them
            for r, res in zip(batch, results):
                r.t_start, r.t_done = t0, t1
                r.future.set_result(res)
            del results, batch
