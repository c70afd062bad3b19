"""The joint stress world (rotating kinematic container, revolute chains, boxes and circles) at a
reduced size: the plain solver against the CPU oracle bit for bit, the coloured one for sanity."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.config5(n_bodies=2048, n_chains=24, half=30.0)


def test_stress_world_plain_matches_oracle(gpu):
    sc = _scene()
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 61):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        if s % 15 == 0:
            assert np.array_equal(w.bodies(0).view(np.uint32), o.bodies().view(np.uint32)), s
            gi, gf = w.contacts(0)
            oi, of = o.contacts()
            assert np.array_equal(gi, oi), s
            assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), s
    w.sync()


def test_stress_world_coloured_stays_sane(gpu):
    sc = _scene()
    w = World(sc)
    w.set_solver("coloured")
    pen = []
    for _ in range(120):
        w.step(DT, VI, PI)
        pen.append(w.max_penetration()[0])
    b = w.bodies(0)
    assert np.all(np.isfinite(b))
    assert max(pen) < 0.5
    # every chain link stays within reach of its neighbour (joints hold)
    links = np.array([j[:2] for j in sc.joints])
    d = np.hypot(b[links[:, 0], 3] - b[links[:, 1], 3], b[links[:, 0], 4] - b[links[:, 1], 4])
    assert d.max() < 2.0
    w.sync()
