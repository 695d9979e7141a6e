"""Replica bookkeeping for multi-GPU runs.

The stencil path has no data-path collective: every rank solves its own
grids (the reference has no multi-GPU code; replicas are the only sharding
that keeps results identical). The only cross-rank step is host-side timing:
the job's time is the slowest rank's, its work the sum of all ranks' work.
"""
from __future__ import annotations

import os


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str):
    """Initialises torch.distributed when launched with more than one rank."""
    import torch.distributed as dist
    _, ws, _ = world()
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend)


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def reduce_max(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(local_work: float, local_seconds: float, device=None) -> tuple[float, float]:
    """(total work over all ranks / slowest rank's time, slowest time)."""
    t = reduce_max(local_seconds, device)
    w = reduce_sum(local_work, device)
    return w / t if t > 0 else 0.0, t
