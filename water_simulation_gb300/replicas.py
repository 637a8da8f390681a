"""Replica aggregation for multi-GPU runs of independent scenes.

The DFSPH step of one scene does not shard across GPUs here (no halo
exchange is built); N GPUs run N independent replicas. The only cross-rank
traffic is this host-side aggregation of the timing: the job time is the
slowest rank's, the work is every rank's particle-steps.
"""
from __future__ import annotations


def aggregate(local_ms: float, local_particle_steps: float, world: int) -> tuple[float, float]:
    """(max milliseconds over ranks, total particle-steps over ranks)."""
    if world <= 1:
        return float(local_ms), float(local_particle_steps)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(local_ms)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(local_particle_steps)], dtype=torch.float64)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def throughput(local_ms: float, local_particle_steps: float, world: int) -> float:
    """Whole-job particle-steps/s: all ranks' work over the slowest rank's time."""
    ms, work = aggregate(local_ms, local_particle_steps, world)
    return work / (ms * 1e-3)
