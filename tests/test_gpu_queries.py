"""World queries on the device (b2World::QueryAABB, closest-hit b2World::RayCast) against the
reference's results on the same stepped scenes (golden vectors from tests/golden/make_golden.py)."""
from __future__ import annotations

import importlib.util
import os

import numpy as np
import pytest

from box2dpp_gb300.world import World
from tests._util import DT, GOLDEN, PI, VI, golden

pytestmark = pytest.mark.gpu


def _scenes():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.query_scenes()


@pytest.mark.parametrize("name,make,steps", _scenes(), ids=[s[0] for s in _scenes()])
def test_queries_match_reference(gpu, name, make, steps):
    g = golden(f"query_{name}")
    w = World(make())
    for _ in range(int(g["steps"])):
        w.step(DT, VI, PI)
    got = w.query_aabb(g["boxes"])
    offs = np.concatenate([[0], np.cumsum(g["counts"])])
    for i, f in enumerate(got):
        assert np.array_equal(f, g["fixtures"][offs[i]:offs[i + 1]]), (name, i)
    fix, hit = w.raycast(g["rays"])
    assert np.array_equal(fix, g["ray_fixture"]), name
    hits = fix >= 0
    assert np.array_equal(hit[hits].view(np.uint32), g["ray_hit"][hits].view(np.uint32)), name
    w.sync()


def test_fixture_queries_match_reference_golden(gpu):
    """b2Fixture::TestPoint, RayCast and GetAABB of every fixture after 60 device steps, bit for bit
    with the reference's results (golden fixture_queries.npz)."""
    import numpy as np

    from box2dpp_gb300 import scenes
    from box2dpp_gb300.world import World
    from tests._util import DT, PI, VI, golden

    g = golden("fixture_queries")
    w = World(scenes.destroy_mix(scenes.SplitMix64(5)))
    for _ in range(int(g["steps"])):
        w.step(DT, VI, PI)
    for q, want in zip(g["queries"], g["outputs"]):
        got = w.fixture_query(int(q[0]), int(q[1]), q[2:])
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (q, got, want)
