"""Replica aggregation across ranks (gloo, world size 2, on CPU): the job
time is the slowest rank's and the rate counts every rank's units."""
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
