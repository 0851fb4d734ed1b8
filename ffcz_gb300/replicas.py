"""Replica aggregation for multi-GPU runs (one independent field per rank).

The corrector does not shard a single field (that would need two all-to-all
transposes per iteration); N GPUs run N independent replicas.  A timed
region is bracketed by barriers and its duration is the maximum over ranks;
the throughput counts every rank's bytes.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def world() -> tuple[int, int]:
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def barrier() -> None:
    if world()[1] > 1:
        dist.barrier()


def max_over_ranks(v: float, device=None) -> float:
    if world()[1] == 1:
        return v
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(bytes_per_rank: float, seconds_per_rank: float, device=None) -> tuple[float, float]:
    """(aggregate bytes/s over all ranks, the max time over ranks)."""
    t = max_over_ranks(seconds_per_rank, device)
    return bytes_per_rank * world()[1] / t, t
