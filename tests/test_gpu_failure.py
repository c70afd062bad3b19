"""Failure paths of the device step, made on the host and ended by bounded device loops (no fault,
trap or hang): a world whose contact slots run out returns GB_ERR_CAPACITY from gb_world_sync, a
world whose time-of-impact events in a step exceed the limit returns GB_ERR_TIMEOUT, and in both cases
the CUDA context stays usable: a new world steps bit-exactly afterwards. With grow-and-retry on, the
same worlds complete every step bit-exactly, the overflowing steps run again with larger buffers."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _context_still_usable():
    sc = scenes.pyramid(6)
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for _ in range(20):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    w.sync()
    assert np.array_equal(w.bodies().view(np.uint32), o.bodies().view(np.uint32))


def test_contact_slots_running_out_reports_capacity(gpu):
    sc = scenes.pyramid(8)  # 36 boxes: about 80 contacts once settled
    w = World(sc)
    w.set_limits(contact_capacity=16)
    for _ in range(30):
        w.step(DT, VI, PI)
    with pytest.raises(_lib.GbError) as e:
        w.sync()
    assert e.value.status == _lib.GB_ERR_CAPACITY
    # the contacts that did fit are the first the reference would create, never more than the slots
    ints, _ = w.contacts()
    assert len(ints) <= 16
    w.close()
    _context_still_usable()


def test_more_new_pairs_than_slots_reports_capacity_at_once(gpu):
    # the first step finds about 90 pairs for 16 free slots
    w = World(scenes.pyramid(8))
    w.set_limits(contact_capacity=16)
    w.step(DT, VI, PI)
    with pytest.raises(_lib.GbError) as e:
        w.sync()
    assert e.value.status == _lib.GB_ERR_CAPACITY


def test_time_of_impact_event_limit_reports_timeout(gpu):
    sc = scenes.drop(400, scenes.SplitMix64(11), allow_sleep=False)  # several events per step
    w = World(sc)
    w.set_limits(max_toi_events=1)
    for _ in range(60):
        w.step(DT, VI, PI)
    with pytest.raises(_lib.GbError) as e:
        w.sync()
    assert e.value.status == _lib.GB_ERR_TIMEOUT
    w.close()
    _context_still_usable()


def test_limits_are_checked(gpu):
    w = World(scenes.pyramid(3))
    with pytest.raises(_lib.GbError):
        w.set_limits(contact_capacity=-1)
    with pytest.raises(_lib.GbError):
        w.set_limits(max_toi_events=0)
    w.step(DT, VI, PI)
    # the contact capacity is fixed once the world is on the device
    with pytest.raises(_lib.GbError):
        w.set_limits(contact_capacity=64)
    w.set_limits(max_toi_events=8)
    w.step(DT, VI, PI)
    w.sync()


def test_recovery_grows_the_contact_slots(gpu):
    sc = scenes.pyramid(8)
    w = World(sc)
    w.set_limits(contact_capacity=16)
    w.set_recovery(6)
    o = oracle.OracleWorld(sc, "port", "project")
    for _ in range(30):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    w.sync()  # no error left
    assert w.recoveries() >= 1
    assert np.array_equal(w.bodies().view(np.uint32), o.bodies().view(np.uint32))
    ints, _ = w.contacts()
    assert len(ints) == len(o.contacts()[0]) > 16


def test_recovery_raises_the_event_limit(gpu):
    sc = scenes.drop(400, scenes.SplitMix64(11), allow_sleep=False)
    w = World(sc)
    w.set_limits(max_toi_events=1)
    w.set_recovery(8)
    o = oracle.OracleWorld(sc, "port", "project")
    for _ in range(60):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    w.sync()
    assert w.recoveries() >= 1
    assert np.array_equal(w.bodies().view(np.uint32), o.bodies().view(np.uint32))
