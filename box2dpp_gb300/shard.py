"""Weak-scaling shards of the batched-worlds workload: one process per GPU, each stepping its own
worlds. The job is one world set of n_worlds per rank, drawn from one seed and partitioned across the
ranks by estimated cost (the sum of the worlds' body counts; largest worlds first, each to the rank
with the least cost so far), so every rank carries about the same work. Worlds are independent, so
the step has no data-path exchange; ranks meet only at a barrier around the timed region and at one
max-reduction of the elapsed time (whole-job throughput = all ranks' bodies x steps / the slowest
rank's time)."""
from __future__ import annotations

import os

def dist_env():
    """(rank, world size, local rank) from the launcher's environment (torch.distributed.run)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def partition_by_cost(costs, n_ranks: int):
    """Indices of the units each rank takes: largest cost first, each to the rank whose total is
    smallest so far (the lowest rank on a tie); every index in exactly one part, each part ascending."""
    totals = [0.0] * n_ranks
    parts = [[] for _ in range(n_ranks)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(n_ranks), key=lambda q: (totals[q], q))
        parts[r].append(i)
        totals[r] += costs[i]
    return [sorted(p) for p in parts]


def shard_workload(n_worlds: int, seed: int, rank: int, allow_sleep: bool = False, world_size: int = 1):
    """The rank's worlds: its part of the job's n_worlds x world_size worlds (one seed), partitioned
    by body count. With one rank this is the whole set, in order."""
    from . import scenes

    specs = scenes.config3_specs(n_worlds * world_size, seed=seed)
    return [scenes.config3_world(specs[i], allow_sleep) for i in shard_indices(specs, rank, world_size)]


def shard_indices(specs, rank: int, world_size: int):
    """Indices into the job's world specs that the rank steps."""
    if world_size <= 1:
        return list(range(len(specs)))
    return partition_by_cost([sp[0] for sp in specs], world_size)[rank]


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
