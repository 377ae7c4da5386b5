"""Replica bookkeeping for runs over several GPUs of one node.

Parameter sets are independent, so N GPUs run N replicas: each rank evaluates
its own slice of sets (its own seeds in the benchmark) with no exchange on the
data path; the only collective is the max over ranks of the timed duration,
and the job's throughput is the units of all ranks over that time (weak
scaling: the work per GPU is fixed as N grows).
"""
from __future__ import annotations

import os
from typing import Tuple


def rank_info() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seeds(rank: int, seed_params: int = 2026, seed_grids: int = 7) -> Tuple[int, int]:
    """Seeds of the rank's slice of the batched workload (a different slice per rank)."""
    return seed_params + rank, seed_grids + rank


def set_range(rank: int, world: int, n_total: int) -> Tuple[int, int]:
    """Contiguous slice [lo, hi) of n_total sets for the rank (sizes differ by at most one)."""
    base, extra = divmod(n_total, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The maximum of x over the ranks of the process group (x itself without one)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, steps: int, world: int, seconds: float) -> float:
    """Units per second of the whole job: every rank's units over the slowest rank's time."""
    return world * units_per_rank * steps / seconds
