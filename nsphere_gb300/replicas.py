"""Replica bookkeeping of a multi-GPU run.

The step of one halo has no exchange that pays on one node, so N GPUs run N
independent halos (one process per GPU, seeds offset by the rank) and a job's rate is
all ranks' particle-steps over the slowest rank's time.  These helpers are what
bench.py does around its timed region; they work with any torch.distributed backend
(NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations

import os


def rank_env() -> tuple[int, int, int]:
    """(rank, local rank, world size) from the torchrun environment (1 process when unset)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The largest of every rank's value (each rank gets it)."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's milliseconds."""
    return units_per_rank * world / (ms_max / 1e3)


def replica_seed(base: int, rank: int) -> int:
    """Seed of rank's halo: independent replicas, reproducible per rank."""
    return base + rank
