"""Destruction between steps on the host mirror of a world that has not been uploaded (no GPU): the
listener calls and the proxy ids of fixtures created afterwards equal the reference's (its
b2DynamicTree hands freed nodes out again last-in first-out), and bad indices are rejected."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes
from box2dpp_gb300.world import World
from tests._util import apply_ops


def _ops():
    box = (3, [0.4, 0.4], 2, 1.0)
    add = lambda x, y, *f: ("add", 2, [x, y, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0], list(f))
    return [("body", 12), ("body", 3), ("joint", 2), ("fixture", 48), ("body", 43), add(-3.0, 14.0, box),
            add(0.0, 14.0, box, box), ("body", 30), add(3.0, 14.0, box), ("body", 0), add(6.0, 14.0, box)]


@pytest.mark.parametrize("kind", ["port"] + (["reference"] if oracle.reference_available() else []))
def test_host_destruction_matches_oracle(kind):
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    g = World(sc)
    o = oracle.OracleWorld(sc, kind, "project")
    assert apply_ops(g, _ops()) == apply_ops(o, _ops())
    gi, gf = g.proxies()
    oi, of = o.proxies()
    assert np.array_equal(gi, oi)
    assert np.array_equal(gf.view(np.uint32), of.view(np.uint32))
    assert np.array_equal(g.bodies().view(np.uint32), o.bodies().view(np.uint32))


def test_bad_destruction_rejected():
    g = World(scenes.destroy_mix(scenes.SplitMix64(5)))
    g.destroy_body(12)
    for call in (lambda: g.destroy_body(12), lambda: g.destroy_body(10_000), lambda: g.destroy_fixture(12),
                 lambda: g.destroy_joint(-1)):
        with pytest.raises(_lib.GbError):
            call()
    g.destroy_joint(0)
    with pytest.raises(_lib.GbError):
        g.destroy_joint(0)
