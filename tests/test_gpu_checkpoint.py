"""World checkpoints between device steps: the steps after a restore are bit for bit those of the world
the checkpoint was taken from, whether restored into a fresh handle, into one world of a batch, or
back into the same handle after it stepped on (rewind); with the reference-order and the coloured
solver, contacts with warm-start impulses, sleeping bodies, joints and a tracked broadphase tree."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, digest

pytestmark = pytest.mark.gpu


def _digests(w, steps, k=0):
    out = []
    for _ in range(steps):
        w.step(DT, VI, PI)
        out.append(bytes(digest(w.bodies(k), *w.contacts(k))))
    return out


@pytest.mark.parametrize("solver", ["plain", "coloured"])
def test_resume_in_a_fresh_handle_is_bit_exact(gpu, solver):
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    a = World(sc)
    a.set_solver(solver)
    for _ in range(60):
        a.step(DT, VI, PI)
    data = a.checkpoint()
    want = _digests(a, 120)
    b = World(scenes.pyramid(2))
    b.set_solver(solver)
    b.restore(data)
    assert _digests(b, 120) == want


def test_rewind_in_the_same_handle(gpu):
    a = World(scenes.drop(300, scenes.SplitMix64(7)))
    for _ in range(40):
        a.step(DT, VI, PI)
    data = a.checkpoint()
    first = _digests(a, 80)
    a.restore(data)
    assert _digests(a, 80) == first


def test_restore_into_one_world_of_a_batch(gpu):
    sc = scenes.joint_zoo(scenes.SplitMix64(6))
    a = World(sc, track_tree=True)
    for _ in range(50):
        a.step(DT, VI, PI)
    data = a.checkpoint()
    want = _digests(a, 100)
    want_tree = a.tree_stats()
    b = World([scenes.pyramid(6), scenes.pyramid(2), scenes.drop(120, scenes.SplitMix64(3))], track_tree=True)
    for _ in range(10):
        b.step(DT, VI, PI)
    other = b.checkpoint(0)
    b.restore(data, 1)
    assert _digests(b, 100, k=1) == want
    assert b.tree_stats(1) == want_tree
    # world 0 stepped on as if nothing happened beside it
    c = World([scenes.pyramid(6)])
    c.restore(other)
    for _ in range(100):
        c.step(DT, VI, PI)
    b.sync()
    c.sync()
    assert np.array_equal(b.bodies(0).view(np.uint32), c.bodies(0).view(np.uint32))


def test_sleeping_world_resumes_bit_exact(gpu):
    a = World(scenes.config1())
    for _ in range(300):
        a.step(DT, VI, PI)
    data = a.checkpoint()
    want = _digests(a, 60)
    b = World(scenes.pyramid(2))
    b.restore(data)
    assert _digests(b, 60) == want
