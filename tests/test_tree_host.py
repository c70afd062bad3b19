"""The host copy of the broadphase tree (b2World::GetTreeHeight, GetTreeBalance, GetTreeQuality) as far
as it runs without a GPU: a world built with tree tracking, then changed between steps (destruction,
SetActive, creation), against the reference's tree (the restatement on hosts without the reference
tree); and the calls' argument rules."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300._lib import BODY_ACTIVE, BODY_TYPE, GB_ERR_INVALID, GbError
from box2dpp_gb300.world import World
from tests._util import apply_ops, destroy_script


def _kind():
    return "reference" if oracle.reference_available() else "port"


def _same(a, b):
    return (a[0], a[1]) == (b[0], b[1]) and np.float32(a[2]).view(np.uint32) == np.float32(b[2]).view(np.uint32)


@pytest.mark.parametrize("name", ["pyramid", "drop300", "config2_10k", "chain_terrain", "sensors"])
def test_built_tree_matches(name):
    sc = {"pyramid": lambda: scenes.config1(), "drop300": lambda: scenes.drop(300, scenes.SplitMix64(7)),
          "config2_10k": lambda: scenes.config2(10000, seed=1, allow_sleep=True),
          "chain_terrain": lambda: scenes.chain_terrain(scenes.SplitMix64(12)),
          "sensors": lambda: scenes.sensors(scenes.SplitMix64(13))}[name]()
    w = World(sc, track_tree=True)
    o = oracle.OracleWorld(sc, _kind(), "project")
    assert _same(w.tree_stats(), o.tree_stats()), (w.tree_stats(), o.tree_stats())


def test_tree_after_host_changes_matches():
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    w = World(sc, track_tree=True)
    o = oracle.OracleWorld(sc, _kind(), "project")
    for _, ops in sorted(destroy_script().items()):
        apply_ops(w, ops)
        apply_ops(o, ops)
        assert _same(w.tree_stats(), o.tree_stats())
    for body, prop, v in [(13, BODY_ACTIVE, 0.0), (44, BODY_ACTIVE, 0.0), (30, BODY_ACTIVE, 0.0), (44, BODY_ACTIVE, 1.0),
                          (13, BODY_ACTIVE, 1.0), (30, BODY_TYPE, 0.0), (30, BODY_ACTIVE, 1.0)]:
        w.body_set(body, prop, v)
        o.body_set(body, prop, v)
        assert _same(w.tree_stats(), o.tree_stats()), (body, prop, v)


def test_tree_calls_argument_rules():
    sc = scenes.config1()
    w = World(sc)
    with pytest.raises(GbError):
        w.tree_stats()  # not tracking
    # the world's proxies exist already: their tree's history is not known
    assert w.lib.gb_world_track_tree(w.h, 1) == GB_ERR_INVALID
    empty = World(scenes.Scene(name="empty"), track_tree=True)
    assert empty.tree_stats() == (0, 0, np.float32(0.0))


def test_shift_origin_before_stepping_matches():
    """b2World::ShiftOrigin on the host: bodies, proxies (ids and fat boxes) and the tree as the
    reference's."""
    sc = scenes.pulley_mouse(scenes.SplitMix64(4))
    w = World(sc, track_tree=True)
    o = oracle.OracleWorld(sc, _kind(), "project")
    for x, y in ((10.0, -3.0), (-25.5, 7.25)):
        w.shift_origin(x, y)
        o.shift_origin(x, y)
    assert np.array_equal(w.bodies().view(np.uint32), o.bodies().view(np.uint32))
    (i1, f1), (i2, f2) = w.proxies(), o.proxies()
    assert np.array_equal(i1, i2) and np.array_equal(f1.view(np.uint32), f2.view(np.uint32))
    assert _same(w.tree_stats(), o.tree_stats())
