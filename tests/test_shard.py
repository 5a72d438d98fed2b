"""Multi-GPU host logic on the CPU: balanced shares of independent jobs, and
the timing / work reductions of a multi-rank run, checked with two `gloo`
ranks (no GPU involved)."""

import os
import socket

import numpy as np
import pytest

from rusterize_gb300.shard import job_cost, shard_jobs


def test_shares_are_a_balanced_partition():
    rng = np.random.default_rng(3)
    costs = [job_cost(int(s), int(s), int(v)) for s, v in zip(np.exp(rng.uniform(np.log(256), np.log(8192), 300)),
                                                             rng.integers(100, 100_000, 300))]
    for world in (1, 2, 3, 8):
        shares = shard_jobs(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))  # every job exactly once
        loads = [sum(costs[i] for i in s) for s in shares]
        assert max(loads) - min(loads) <= max(costs)  # greedy bound: within one job
        assert all(s == sorted(s) for s in shares)
    assert shard_jobs([], 4) == [[], [], [], []]
    assert shard_jobs([5.0, 1.0, 1.0], 2) == [[0], [1, 2]]
    with pytest.raises(ValueError):
        shard_jobs([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    from rusterize_gb300 import shard

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        r, w, local = shard.dist_env()
        costs = [float(10 + (i * 7919) % 101) for i in range(57)]
        mine = shard.shard_jobs(costs, w)[r]
        shard.barrier()
        t = shard.max_over_ranks(1.5 + r)  # a step time
        units = shard.sum_over_ranks(float(len(mine)))
        q.put((r, local, mine, t, units))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_jobs_and_reduce_timing():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, l0, m0, t0, u0), (r1, l1, m1, t1, u1) = res
    assert (r0, l0, r1, l1) == (0, 0, 1, 1)
    assert sorted(m0 + m1) == list(range(57)) and not set(m0) & set(m1)
    assert t0 == t1 == 2.5  # the slowest rank's time on every rank
    assert u0 == u1 == 57.0


def test_row_bands_cover_rows_once_and_balance_cost():
    from rusterize_gb300.shard import row_bands

    for nrows in (0, 1, 7, 1000):
        for world in (1, 2, 3, 8):
            bands = row_bands(nrows, world)
            assert len(bands) == world and bands[0][0] == 0 and bands[-1][1] == nrows
            assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
            assert all(r0 <= r1 for r0, r1 in bands)
    cost = np.zeros(1000)
    cost[900:] = 1.0  # all the work in the last 100 rows
    bands = row_bands(1000, 4, cost)
    assert bands[0][0] == 0 and bands[-1][1] == 1000
    loads = [cost[r0:r1].sum() for r0, r1 in bands]
    assert max(loads) <= 26 and bands[0][1] >= 900
    with pytest.raises(ValueError):
        row_bands(10, 2, np.ones(9))


def _row_split_main(rank, world, port, q):
    import torch.distributed as dist

    import rusterize_gb300 as rz
    from rusterize_gb300 import shard, synth
    from _util import oracle_burn

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        a, _ = synth.mixed(seed=11, scale=0.0004)
        info = rz.raster_info(a.table, res=(1.25, 0.8), extent=a.extent)
        lo, hi = shard.geometry_rows(a.table, info)
        # rows weighted by the geometries that can touch them
        cost = np.zeros(info.nrows + 3)
        np.add.at(cost, np.clip(lo, -1, info.nrows) + 1, 1.0)
        np.add.at(cost, np.clip(hi, -1, info.nrows) + 2, -1.0)
        row_cost = np.cumsum(cost)[1:info.nrows + 1]
        r0, r1 = shard.row_bands(info.nrows, world, row_cost)[rank]
        idx = shard.select_rows(a.table, info, r0, r1)
        assert (np.diff(idx) > 0).all()  # input order kept
        sub = a.table.select(idx)
        vals = (np.arange(a.table.n_geoms) % 7 + 1).astype(np.float64)
        mine = oracle_burn(sub, info, fn="sum", values=vals[idx], background=0.0, dtype="float64")[:, r0:r1]
        parts = [None] * world
        dist.all_gather_object(parts, (r0, r1, len(idx), mine))
        if rank == 0:
            whole = oracle_burn(a.table, info, fn="sum", values=vals, background=0.0, dtype="float64")
            parts.sort(key=lambda t: t[0])
            joined = np.concatenate([p[3] for p in parts], axis=1)
            q.put((True, whole.shape == joined.shape and np.array_equal(whole, joined),
                   [(p[0], p[1], p[2]) for p in parts], a.table.n_geoms))
        else:
            q.put((False, None, None, None))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_the_rows_of_one_job():
    """Each rank burns its row band of the same job from the geometries that
    can write there (with the oracle, on the CPU); the gathered bands equal
    the whole burn, so no geometry that writes in a band was dropped and the
    write order was kept."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_row_split_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (is0, equal, bands, n) = next(r for r in res if r[0])
    assert equal
    assert bands[0][0] == 0 and bands[0][1] == bands[1][0]
    assert 0 < bands[0][2] < n and 0 < bands[1][2] < n  # each rank burns a proper subset
