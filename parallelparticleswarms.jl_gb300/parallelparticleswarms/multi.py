"""One process per GPU: the rank bookkeeping of the multi-GPU bench path.

The synchronous step shards by whole swarms: every rank solves an independent
swarm on its own GPU (weak scaling), so no collective touches the data path.
The only exchange is the timing reduction: the job's time is the slowest
rank's, and its throughput counts the particle-iterations of every rank.
"""
from __future__ import annotations

import os


def rank_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def swarm_seed(base: int, rank: int) -> int:
    """Seed of the rank's swarm: ranks draw disjoint Philox streams."""
    return (base + 1000 * rank) & 0xFFFFFFFFFFFFFFFF


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The largest `value` over all ranks (the job's time is the slowest rank's)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, slowest_ms: float) -> float:
    """Whole-job rate: the units of every rank over the slowest rank's time."""
    return units_per_rank * world / (slowest_ms / 1000.0)
