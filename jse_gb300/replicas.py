"""Multi-GPU form of the evaluation path: independent replicas, one process per GPU.

Atoms are independent once the neighbour list exists and structures of a batch are
independent, so the path needs no collective on its data: every rank evaluates its own
structures on its own GPU.  The only cross-rank steps are host-side bookkeeping: a
barrier around the timed region, the maximum of the ranks' times, and the whole-job
rate (units of all ranks over that maximum).  ``shard`` splits a list of independent
structures between ranks when a caller wants data-parallel rather than replicated work.
"""
from __future__ import annotations

from typing import Optional, Sequence


def shard(items: Sequence, rank: int, world: int) -> list:
    """Items of ``rank`` out of ``world``: every ``world``-th item from ``rank`` on."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must lie in [0, world)")
    return list(items[rank::world])


def barrier(dist=None):
    if dist is not None:
        dist.barrier()


def max_over_ranks(seconds: float, dist=None) -> float:
    """Largest of the ranks' timings (the job is as slow as its slowest rank)."""
    if dist is None:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def whole_job_rate(units_per_rank_step: int, steps: int, world: int, t_max: float) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    if t_max <= 0.0:
        raise ValueError("timed region must be positive")
    return units_per_rank_step * steps * world / t_max


def init_from_env(backend: str = "gloo"):
    """Join the process group named by torchrun's environment (None with one process)."""
    import os
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 1
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist, dist.get_rank(), dist.get_world_size()
