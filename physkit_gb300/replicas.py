"""Multi-GPU form of the batched world step: replicas, one rank per GPU, no data-path collective.

Worlds are independent, so a batch shards by world: rank r steps its own batch (scene seed + r) and
the ranks meet only around the timed region — a barrier before it, and the maximum of the ranks'
device times after it. The job's throughput is the sum of the ranks' bodies x steps over that
maximum.
"""
from __future__ import annotations


def rank_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s batch: each rank simulates different worlds."""
    return base + rank


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The largest `value` over all ranks (the job's time); `value` itself without a process group.
    `device` is where the reduction tensor lives: "cuda" under NCCL, "cpu" under gloo."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """Sum of `value` over all ranks (each rank's batch has its own body count)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(units_all_ranks: float, steps: int, ms_max: float) -> float:
    """Units (bodies) x steps of all ranks per second of the slowest rank's timed region."""
    return units_all_ranks * steps / (ms_max / 1e3)
