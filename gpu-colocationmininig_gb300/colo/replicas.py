"""Replicas across GPUs: one independent mining process per GPU.

The path has no exchange step (independent jobs shard with no collective),
so N GPUs run N replicas.  A timed run is bracketed by a barrier and device
synchronisation on every rank; the aggregate is the units all ranks
processed divided by the slowest rank's time.
"""
from __future__ import annotations


def aggregate(dist, units: float, ms: float, device=None):
    """(sum of `units` over ranks, max of `ms` over ranks); identity without a process group."""
    if dist is None:
        return float(units), float(ms)
    import torch

    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    m = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())


def throughput(dist, units: float, ms: float, device=None) -> float:
    """Whole-job units per second: all ranks' units over the slowest rank's time."""
    total, slowest = aggregate(dist, units, ms, device)
    return total / (slowest / 1e3) if slowest > 0 else 0.0
