"""Replica aggregation and instance sharding across ranks (gloo, world size
2, on CPU): the job time is the slowest rank's, the rate counts every rank's
units, and a sharded batch of instances covers every instance exactly once
with per-instance results equal to a single-rank run."""
import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from bsam.replicas import job_rate, job_time
    local = 2.0 + 3.0 * rank                 # rank 1 is the slow one
    t = job_time(local, dist)
    rate, t2 = job_rate(10, local, dist)
    q.put((rank, t, rate, t2))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks():
    import multiprocessing as mp
    import socket
    ctx = mp.get_context('spawn')
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate, t2 in out:
        assert t == 5.0 and t2 == 5.0
        assert rate == pytest.approx(2 * 10 / 5.0)


def test_single_process_rate():
    from bsam.replicas import job_rate
    assert job_rate(7, 2.0) == (3.5, 2.0)


def _instance_result(i):
    """One seeded instance of the batched workload, root level only (small
    enough for the CPU): V-cycles and residual history on the oracle."""
    import warnings
    from bsam import ebOptions
    from bsam.instances import random_elliptic
    from bsam.solve import build_hierarchy
    from bsam.flat import flatten
    from bsam_oracle import OracleBackend, OracleHier
    prob, o = random_elliptic(1000 + i)
    o = dict(o, BaseCells=32, MaxLevels=1)
    opts = ebOptions(o)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        H = build_hierarchy(prob, opts, OracleBackend())
    fl = flatten(H)
    it, hist, rel, vis = OracleHier(fl, opts).solve_cycles(opts.MaxVCycles + 2)
    return i, it, hist.tobytes(), rel


def _shard_worker(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from bsam.replicas import shard, gather, job_rate_units
    mine = [_instance_result(i) for i in shard(n, rank, world)]
    everyone = gather(mine, dist)
    rate, t = job_rate_units(len(mine), 1.0 + rank, dist)
    q.put((rank, everyone, rate, t))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_instance_shards_cover_each_instance_once():
    import multiprocessing as mp
    import socket
    n = 5
    ctx = mp.get_context('spawn')
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    q = ctx.Queue()
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted((q.get(timeout=300) for _ in ps), key=lambda r: r[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    alone = {r[0]: r for r in (_instance_result(i) for i in range(n))}
    for rank, everyone, rate, t in out:
        got = [r for part in everyone for r in part]
        assert sorted(r[0] for r in got) == list(range(n))      # every instance exactly once
        for r in got:
            assert r == alone[r[0]]                              # same result as the single-rank run
        assert t == 2.0 and rate == pytest.approx(n / 2.0)      # all units over the slowest rank's time


def test_shard_split():
    from bsam.replicas import shard
    assert shard(7, 0, 3) == [0, 3, 6] and shard(7, 1, 3) == [1, 4] and shard(7, 2, 3) == [2, 5]
    assert shard(4) == [0, 1, 2, 3]
    with pytest.raises(ValueError):
        shard(4, 2, 2)
