"""Replica bookkeeping of the multi-GPU benchmark.

Pixels, samples and requests are independent, so N GPUs run N replicas: one process per
GPU renders its own image with its own seed and nothing is exchanged between them. The
job's time is the slowest rank's, and its throughput counts the work of every rank.
"""
import os


def rank_world_local():
    """(RANK, WORLD_SIZE, LOCAL_RANK) as torchrun sets them; (0, 1, 0) when run alone."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base_seed: int, rank: int) -> int:
    """Each replica's random-stream seed: distinct images, no shared samples."""
    return base_seed + rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest value over all ranks (the job's time); `dist` is torch.distributed
    with an initialised process group, or None when running alone."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job units per second: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds
