"""Replicas and instance shards across GPUs.

One hierarchy does not shard (a level's patches would need a ghost
exchange after every colour), so N GPUs run N independent replicas, one
process per GPU, with no data-path collective.  Independent instances (a
batch of elliptic problems, served requests) shard by instance: each rank
takes every world-th instance and solves its share as its own batch.  The
only cross-rank steps are the timing -- the job's time is the slowest
rank's, and its throughput is the units all ranks processed over that time
-- and, after the timed region, gathering per-instance results for the
report.
"""
from __future__ import annotations


def job_time(local, dist=None, device=None):
    """Max of a per-rank time over all ranks (local value without dist)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local)
    import torch
    t = torch.tensor([float(local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, local_seconds, dist=None, device=None):
    """Whole-job throughput: units of every rank over the slowest rank's time."""
    world = dist.get_world_size() if (dist is not None and dist.is_initialized()) else 1
    t = job_time(local_seconds, dist, device)
    return world * units_per_rank / t, t


def shard(n, rank=0, world=1):
    """Instance indices of one rank: every world-th of 0..n-1, starting at
    its rank (each index on exactly one rank; shares differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f'bad rank {rank} of {world}')
    return list(range(rank, n, world))


def job_rate_units(local_units, local_seconds, dist=None, device=None):
    """Whole-job throughput when ranks process different numbers of units:
    the sum of every rank's units over the slowest rank's time."""
    t = job_time(local_seconds, dist, device)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(local_units) / t, t
    import torch
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()) / t, t


def gather(obj, dist=None):
    """Every rank's `obj` in rank order (outside any timed region)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out
