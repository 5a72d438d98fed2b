"""The burn server (rusterize_gb300/serve.py): admission by device-memory
budget on the CPU, and on the GPU continuous batching whose every result is
the same raster as the job burned alone."""

import threading
import time
from concurrent.futures import Future

import numpy as np
import pytest

from rusterize_gb300.serve import Admission, Request


def _req(nbytes, dtype="float32"):
    return Request(job=None, dtype=dtype, nbytes=nbytes, future=Future(), t_submit=time.perf_counter())


# ---------------------------------------------------------------- CPU ------
def test_admission_takes_the_oldest_dtype_in_order_within_the_budget():
    a = Admission(budget_bytes=100, max_batch=10)
    reqs = [_req(30), _req(30, "uint8"), _req(30), _req(30), _req(5, "uint8")]
    for r in reqs:
        a.put(r)
    b1 = a.take()
    assert b1 == [reqs[0], reqs[2], reqs[3]] and a.reserved == 90
    # the uint8 head does not fit (90 + 30 > 100): nothing is taken until a release
    assert a.take(timeout=0.05) == []
    a.release(30)
    b2 = a.take()
    assert b2 == [reqs[1], reqs[4]] and a.reserved == 95
    assert a.peak_reserved == 95
    a.close()
    assert a.take() == []


def test_admission_cancel_pending_keeps_reservations_of_taken_batches():
    a = Admission(budget_bytes=100, max_batch=10)
    reqs = [_req(60), _req(60), _req(10, "uint8")]
    for r in reqs:
        a.put(r)
    assert a.take() == [reqs[0]] and a.reserved == 60
    gone = a.cancel_pending()
    assert gone == [reqs[1], reqs[2]] and len(a) == 0
    assert a.reserved == 60  # the running batch still holds its bytes
    a.release(60)
    assert a.take(timeout=0.05) == [] and a.reserved == 0


def test_admission_rejects_requests_beyond_the_budget_and_after_close():
    a = Admission(budget_bytes=100, max_batch=10)
    with pytest.raises(ValueError, match="budget"):
        a.put(_req(101))
    a.close()
    with pytest.raises(RuntimeError, match="closed"):
        a.put(_req(1))


def test_admission_batch_cap_and_blocking_take():
    a = Admission(budget_bytes=1000, max_batch=3)
    for _ in range(5):
        a.put(_req(10))
    assert len(a.take()) == 3 and len(a.take()) == 2
    got = []
    t = threading.Thread(target=lambda: got.append(a.take()))
    t.start()
    time.sleep(0.05)
    assert not got  # blocks while nothing is queued
    r = _req(10)
    a.put(r)
    t.join(5)
    assert got == [[r]]


def test_admission_take_costs_the_requests_it_looks_at_not_the_backlog():
    """A server that has fallen behind holds a backlog of hundreds of thousands
    of requests; one take at one request per batch must not copy it.  20,000
    takes from a 200,000-request backlog finish in well under the time one
    copy of the backlog per take would need (4e9 element moves), and the
    skipped requests of the other dtype keep their place at the front."""
    a = Admission(budget_bytes=1 << 40, max_batch=1)
    reqs = [_req(1, "uint8" if i % 2 else "float32") for i in range(200_000)]
    for r in reqs:
        a.put(r)
    t0 = time.perf_counter()
    out = []
    for _ in range(20_000):
        out.extend(a.take(timeout=0))
    assert time.perf_counter() - t0 < 5.0
    assert out == reqs[:20_000]  # alternating dtypes: the head is always the oldest request
    assert len(a) == 180_000
    a2 = Admission(budget_bytes=1 << 40, max_batch=2)
    rs = [_req(1), _req(1, "uint8"), _req(1, "uint8"), _req(1), _req(1, "uint8")]
    for r in rs:
        a2.put(r)
    assert a2.take(timeout=0) == [rs[0], rs[3]]
    assert a2.take(timeout=0) == [rs[1], rs[2]]
    assert a2.take(timeout=0) == [rs[4]]


# ---------------------------------------------------------------- GPU ------
@pytest.mark.gpu
def test_server_results_equal_single_burns_and_batches_form():
    torch = pytest.importorskip("torch")
    import rusterize_gb300 as rz
    from rusterize_gb300 import synth
    from rusterize_gb300.device import DeviceTable, upload
    from rusterize_gb300.engine import BatchJob, rasterize_table
    from rusterize_gb300.serve import BurnServer

    ws = synth.batch_jobs(seed=77, n_jobs=40, side_range=(64.0, 900.0), max_polygons=800)
    jobs, host = [], []
    for i, w in enumerate(ws):
        dtype = "float32" if i % 3 else "uint8"
        vals = w.values if dtype == "float32" else (w.values * 200).astype(np.uint8)
        info = rz.raster_info(w.table, res=w.res, extent=w.extent)
        bg = w.background if dtype == "float32" else 0
        jobs.append((BatchJob(DeviceTable.upload(w.table), info, upload(vals), w.fn, bg), dtype))
        host.append(rasterize_table(w.table, info, values=vals, fn=w.fn, background=bg, dtype=dtype))
    with BurnServer(budget_bytes=1 << 30, streams=2) as srv:
        futs = [srv.submit(j, dtype=d) for j, d in jobs]
        results = [f.result(timeout=120) for f in futs]
        for (j, d), r, want in zip(jobs, results, host):
            got = r.out.cpu().numpy().view(np.dtype(d)).reshape(want.shape)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
            r.release()
        assert srv.jobs_done == 40 and srv.batches < 40  # arrivals while a batch ran were batched
        assert max(r.batch_jobs for r in results) > 1
        assert srv.admission.reserved == 0


@pytest.mark.gpu
def test_server_backpressure_and_failed_batches():
    torch = pytest.importorskip("torch")
    import rusterize_gb300 as rz
    from rusterize_gb300 import synth
    from rusterize_gb300.device import DeviceTable
    from rusterize_gb300.engine import BatchJob
    from rusterize_gb300.serve import BurnServer

    ws = synth.batch_jobs(seed=78, n_jobs=12, side_range=(200.0, 400.0), max_polygons=200)
    jobs = [BatchJob(DeviceTable.upload(w.table), rz.raster_info(w.table, res=w.res, extent=w.extent), None, w.fn,
                     w.background) for w in ws]
    biggest = max(j.info.nrows * j.info.ncols * 4 for j in jobs)
    with BurnServer(budget_bytes=2 * biggest, streams=2) as srv:
        # the client releases each result as it arrives; the budget never holds more than two rasters
        futs = [srv.submit(j) for j in jobs]
        for f in futs:
            f.result(timeout=120).release()
        assert srv.admission.peak_reserved <= 2 * biggest
        # a request whose table is broken fails its batch; the server keeps serving
        bad = BatchJob(DeviceTable.upload(ws[0].table), jobs[0].info, None, "sum", 0.0)
        bad.table.tensors["part_offsets"][-1] += 1
        fb = srv.submit(bad)
        with pytest.raises(ValueError, match="job"):
            fb.result(timeout=120)
        ok = srv.submit(jobs[1]).result(timeout=120)
        ok.release()
        assert srv.admission.reserved == 0


def test_admission_invariants_under_random_traffic():
    """Random puts, takes and releases: reservations never exceed the budget,
    every request leaves exactly once, and requests of one dtype leave in
    arrival order."""
    hypothesis = pytest.importorskip("hypothesis")
    st = hypothesis.strategies

    ops = st.lists(st.one_of(
        st.tuples(st.just("put"), st.integers(1, 60), st.sampled_from(["float32", "uint8"])),
        st.tuples(st.just("take"), st.just(0), st.just("")),
        st.tuples(st.just("release"), st.just(0), st.just("")),
    ), max_size=80)

    @hypothesis.settings(max_examples=300, deadline=None)
    @hypothesis.given(ops, st.integers(60, 200), st.integers(1, 8))
    def run(seq, budget, max_batch):
        a = Admission(budget_bytes=budget, max_batch=max_batch)
        held, order, out = [], {}, []
        for op, nbytes, dtype in seq:
            if op == "put":
                r = _req(nbytes, dtype)
                order.setdefault(dtype, []).append(r)
                a.put(r)
            elif op == "take":
                b = a.take(timeout=0)
                assert len(b) <= max_batch and len({r.dtype for r in b}) <= 1
                held.extend(b)
                out.extend(b)
            elif held:
                a.release(held.pop(0).nbytes)
            assert a.reserved == sum(r.nbytes for r in held) <= budget
        while held:  # drain: release everything, take the rest
            a.release(held.pop().nbytes)
        while len(a):
            b = a.take(timeout=0)
            out.extend(b)
            for r in b:
                a.release(r.nbytes)
        assert sorted(map(id, out)) == sorted(id(r) for rs in order.values() for r in rs)
        for dtype, rs in order.items():
            assert [r for r in out if r.dtype == dtype] == rs

    run()
