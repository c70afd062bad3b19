"""The sharded workload on the product path: the worlds each rank's part holds step on the GPU to
the same bits as in the whole world set (worlds are independent, so sharding changes no result).
The ranks are stepped one after the other in this process; no kernel waits on another rank."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes, shard
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _state(w, i):
    ints, flts = w.contacts(i)
    return w.bodies(i).view(np.uint32).copy(), ints.copy(), flts.view(np.uint32).copy()


@pytest.mark.parametrize("solver", ["plain", "coloured"])
def test_rank_parts_step_like_the_whole_set(gpu, solver):
    per_rank, ranks, seed = 12, 2, 5
    whole = World(shard.shard_workload(per_rank * ranks, seed, 0))
    whole.set_solver(solver)
    whole.upload()
    for _ in range(40):
        whole.graph_step(DT, VI, PI)
    whole.sync()
    specs = scenes.config3_specs(per_rank * ranks, seed=seed)
    covered = []
    for r in range(ranks):
        part = World(shard.shard_workload(per_rank, seed, r, world_size=ranks))
        part.set_solver(solver)
        part.upload()
        for _ in range(40):
            part.graph_step(DT, VI, PI)
        part.sync()
        idx = shard.shard_indices(specs, r, ranks)
        assert len(idx) == part.n_worlds
        for i, j in enumerate(idx):
            for a, b in zip(_state(part, i), _state(whole, j)):
                assert np.array_equal(a, b), (r, i, j)
        covered += idx
        part.close()
    assert sorted(covered) == list(range(per_rank * ranks))
