"""The N > 1 path of the batched workload on CPU: two gloo ranks, each stepping its part of one world
set with the CPU oracle (no GPU), aggregated the way bench.py aggregates its ranks; the cost
partition covers every world once and balances the ranks' body counts."""
from __future__ import annotations

import os
import socket

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world_size, port, out):
    import sys
    import time

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import oracle
    from box2dpp_gb300 import shard

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    from box2dpp_gb300 import scenes

    worlds = shard.shard_workload(3, seed=1, rank=rank, world_size=world_size)
    names = shard.shard_indices(scenes.config3_specs(3 * world_size, seed=1), rank, world_size)
    bodies = sum(w.dynamic_count for w in worlds)
    ws = [oracle.OracleWorld(w, "port", "project") for w in worlds]
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(3):
        for w in ws:
            w.step()
    el = time.perf_counter() - t0
    dist.barrier()
    rate = shard.whole_job_rate(bodies, 3, el, world_size)
    slowest = shard.max_over_ranks(el, world_size)
    total = shard.sum_over_ranks(bodies, world_size)
    digest = float(sum(float(np.abs(w.bodies()[:, :2]).sum()) for w in ws))
    out[rank] = (names, bodies, el, rate, slowest, total, digest)
    dist.destroy_process_group()


def test_two_rank_shards_are_disjoint_and_aggregate():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
        assert p.exitcode == 0
    r0, r1 = out[0], out[1]
    assert sorted(r0[0] + r1[0]) == list(range(6))             # every world on exactly one rank
    assert r0[5] == r1[5] == r0[1] + r1[1]                     # bodies summed over ranks
    assert r0[4] == r1[4] == max(r0[2], r1[2])                 # slowest rank's time
    assert abs(r0[3] - (r0[1] + r1[1]) * 3 / max(r0[2], r1[2])) < 1e-6 * r0[3]
    assert r0[3] == r1[3]


def _shard():
    import sys

    sys.path.insert(0, ROOT)
    from box2dpp_gb300 import shard

    return shard


def test_partition_covers_each_world_once_and_balances():
    from box2dpp_gb300 import scenes

    shard = _shard()
    specs = scenes.config3_specs(4 * 512, seed=1)
    costs = [sp[0] for sp in specs]
    for n in (1, 2, 4, 8):
        parts = shard.partition_by_cost(costs, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        assert all(p == sorted(p) for p in parts)
        loads = [sum(costs[i] for i in p) for p in parts]
        # greedy largest-first: the spread is at most the largest single cost
        assert max(loads) - min(loads) <= max(costs)
        assert max(loads) <= sum(costs) / n * 1.01


def test_partition_is_deterministic_with_ties_to_the_lowest_rank():
    shard = _shard()
    assert shard.partition_by_cost([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]
    assert shard.partition_by_cost([1, 9, 4, 4], 2) == [[1], [0, 2, 3]]
    assert shard.partition_by_cost([], 3) == [[], [], []]


def test_one_rank_is_the_whole_world_set_in_order():
    from box2dpp_gb300 import scenes

    shard = _shard()
    assert [w.name for w in shard.shard_workload(40, 3, 0)] == [w.name for w in scenes.config3(40, seed=3, allow_sleep=False)]
    a = [w.name for w in shard.shard_workload(20, 3, 1, world_size=2)]
    b = [w.name for w in shard.shard_workload(20, 3, 1, world_size=2)]
    c = [w.name for w in shard.shard_workload(20, 3, 0, world_size=2)]
    assert a == b and a != c
