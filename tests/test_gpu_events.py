"""Listener calls recorded on the device against the CPU oracle's, call for call (kinds, fixtures,
PostSolve impulses bit for bit), for single worlds and a batch."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _compare(sc_list, steps):
    w = World(sc_list)
    w.set_events(True)
    os_ = [oracle.OracleWorld(sc, "port", "project") for sc in sc_list]
    for o in os_:
        o.record_events(True)
    kinds = np.zeros(4, dtype=np.int64)
    for s in range(1, steps + 1):
        w.step(DT, VI, PI)
        for i, o in enumerate(os_):
            o.step(DT, VI, PI)
            gr, gi = w.events(i)
            orr, oi = o.events()
            assert len(gr) == len(orr), (s, i, len(gr), len(orr))
            assert np.array_equal(gr[:, :3], orr), (s, i)
            assert np.array_equal(gi.view(np.uint32), oi.view(np.uint32)), (s, i)
            kinds += np.bincount(gr[:, 0], minlength=4) if len(gr) else 0
    w.sync()
    return kinds


def test_events_single_worlds(gpu):
    for sc in (scenes.pyramid(8), scenes.drop(150, scenes.SplitMix64(41))):
        kinds = _compare([sc], 90)
        assert kinds[0] > 0 and kinds[2] > 0 and kinds[3] > 0, (sc.name, kinds)
    # hanging chains that touch nothing: no calls at all, on both sides
    assert _compare([scenes.chains(3, 6, scenes.SplitMix64(2))], 60).sum() == 0


def test_events_sensors(gpu):
    """Sensor fixtures: begin and end calls of sensor contacts (static zones, proximity circles on
    dynamic bodies, a kinematic sweeper), no pre-solve or post-solve for them."""
    kinds = _compare([scenes.sensors(scenes.SplitMix64(13))], 200)
    assert kinds[0] > 0 and kinds[1] > 0, kinds


def test_events_batch(gpu):
    kinds = _compare(scenes.config3(12, seed=21), 60)
    assert kinds.min() > 0, kinds  # begin, end, pre-solve and post-solve all occur
