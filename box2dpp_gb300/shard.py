"""Weak-scaling shards of the batched-worlds workload: one process per GPU, each stepping its own
worlds. Worlds are independent, so the step has no data-path exchange; ranks meet only at a barrier
around the timed region and at one max-reduction of the elapsed time (whole-job throughput = all
ranks' bodies x steps / the slowest rank's time)."""
from __future__ import annotations

import os

RANK_SEED_STRIDE = 1000003


def dist_env():
    """(rank, world size, local rank) from the launcher's environment (torch.distributed.run)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def rank_seed(seed: int, rank: int) -> int:
    """Seed of a rank's shard: disjoint world sets per rank, reproducible per (seed, rank)."""
    return seed + RANK_SEED_STRIDE * rank


def shard_workload(n_worlds: int, seed: int, rank: int, allow_sleep: bool = False):
    """The rank's worlds: n_worlds of the batched workload drawn from its own seed."""
    from . import scenes

    return scenes.config3(n_worlds, seed=rank_seed(seed, rank), allow_sleep=allow_sleep)


def max_over_ranks(x: float, world_size: int, device=None) -> float:
    """Maximum of x over all ranks (x itself on a single rank)."""
    if world_size <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world_size: int, device=None) -> float:
    if world_size <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(bodies_per_rank: float, steps: int, seconds_per_rank: float, world_size: int, device=None) -> float:
    """Body-steps per second of the whole job: every rank's bodies over the slowest rank's time."""
    total = sum_over_ranks(bodies_per_rank, world_size, device)
    slowest = max_over_ranks(seconds_per_rank, world_size, device)
    return total * steps / slowest
