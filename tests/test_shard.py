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
