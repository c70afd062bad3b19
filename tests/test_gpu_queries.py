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
