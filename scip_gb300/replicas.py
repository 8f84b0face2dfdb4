"""Replicas-only multi-GPU mode.

Branch-and-bound nodes and distinct instances are independent, so N GPUs run N replicas of the batched
propagator on disjoint work with no collective on the data path; only the bench's timing is reduced
(maximum step time over ranks) and throughput is the work of all ranks over that time.  One process per GPU,
launched by torch.distributed.run; NCCL on GPUs, gloo on CPU for tests.
"""
from __future__ import annotations

import os
from typing import Tuple


def rank_env() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment; (0, 1, 0) without it."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def split(total: int, world: int, rank: int) -> range:
    """Contiguous share of `total` work items for `rank` (sizes differ by at most one)."""
    lo = total * rank // world
    hi = total * (rank + 1) // world
    return range(lo, hi)


def node_seed(base: int, rank: int) -> int:
    """Seed of a rank's own node batch (weak scaling: every rank propagates its own full batch)."""
    return base + 1000 * rank


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the process group (the slowest rank sets the step time)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(items_per_rank: int, world: int, step_ms_max: float) -> float:
    """Whole-job throughput: the work of all ranks over the slowest rank's step time."""
    return world * items_per_rank / (step_ms_max / 1e3)
