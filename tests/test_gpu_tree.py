"""b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality of device worlds that track their tree:
after every step, equal to the reference's (golden tree_stats.npz) on trajectories with time-of-impact
events, joints, chains and sensors, a 10,000-body drop, and the destruction and body-property scripts;
the same through graph replay and for one world of a batch."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, golden, tree_cases, tree_stats_mismatch

pytestmark = pytest.mark.gpu

CASES = tree_cases()


@pytest.mark.parametrize("case", [c[0] for c in CASES])
def test_tree_stats_match_reference(gpu, case):
    name, make, steps, script = next(c for c in CASES if c[0] == case)
    w = World(make(), track_tree=True)
    assert tree_stats_mismatch(w, steps, script, golden("tree_stats"), name) is None


def test_tree_stats_through_graph_replay(gpu):
    g = golden("tree_stats")
    w = World(scenes.drop(300, scenes.SplitMix64(7)), track_tree=True)
    hb, q = g["drop300_hb"], g["drop300_quality"]
    for s in range(1, 121):
        w.graph_step(DT, VI, PI)
        h, b, qq = w.tree_stats()
        assert (h, b) == tuple(int(x) for x in hb[s - 1]) and np.float32(qq).view(np.uint32) == q[s - 1].view(np.uint32), s


def test_tree_stats_in_a_batch(gpu):
    g = golden("tree_stats")
    w = World([scenes.pyramid(6), scenes.config1(), scenes.drop(300, scenes.SplitMix64(7))], track_tree=True)
    for s in range(1, 101):
        w.step(DT, VI, PI)
        for k, name in ((1, "pyramid20"), (2, "drop300")):
            h, b, qq = w.tree_stats(k)
            assert (h, b) == tuple(int(x) for x in g[f"{name}_hb"][s - 1]), (s, k)
            assert np.float32(qq).view(np.uint32) == g[f"{name}_quality"][s - 1].view(np.uint32), (s, k)
