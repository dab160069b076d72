"""Replicas across GPUs.

One hierarchy does not shard (a level's patches would need a ghost
exchange after every colour), so N GPUs run N independent replicas, one
process per GPU, with no data-path collective.  The only cross-rank step is
the timing: the job's time is the slowest rank's, and its throughput is the
units all ranks processed over that time.
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
