"""b2Body state changes between steps through gb_body_edits on the GPU against the CPU oracle (which
matches the reference's own b2Body methods, tests/test_oracle_edits.py), bit for bit after every
step; and the edits of a batch land in the right world."""
import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, digest, edit_scene, edit_script, mouse_script

pytestmark = pytest.mark.gpu


def test_gpu_edits_match_oracle(gpu):
    sc = edit_scene()
    script = edit_script()
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 341):
        edits = script.get(s, [])
        for (op, body, vals, wake) in edits:
            o.body_edit(op, body, vals, wake)
        if edits:
            w.body_edits([(0, body, op, vals, wake) for (op, body, vals, wake) in edits])
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        gb, ob = w.bodies(), o.bodies()
        assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ at step {s}"
        gi, gf = w.contacts()
        oi, of = o.contacts()
        assert np.array_equal(digest(gb, gi, gf), digest(ob, oi, of)), f"contacts differ at step {s}"
    w.sync()


def test_gpu_mouse_targets_match_oracle(gpu):
    """Mouse joint targets moved through gb_body_edits, against the CPU oracle (which matches the
    reference's b2MouseJoint::SetTarget) bit for bit every step; a target edit for a joint that is
    not a mouse joint is refused."""
    sc = scenes.pulley_mouse(scenes.SplitMix64(4))
    script = mouse_script()
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 361):
        edits = script.get(s, [])
        for (op, body, vals, wake) in edits:
            o.body_edit(op, body, vals, wake)
        if edits:
            w.body_edits([(0, body, op, vals, wake) for (op, body, vals, wake) in edits])
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        gb, ob = w.bodies(), o.bodies()
        assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ at step {s}"
        gi, gf = w.contacts()
        oi, of = o.contacts()
        assert np.array_equal(digest(gb, gi, gf), digest(ob, oi, of)), f"contacts differ at step {s}"
    for bad in [(0, 0, "mouse_target", (1.0, 1.0), True), (0, 4, "mouse_target", (1.0, 1.0), True)]:
        with pytest.raises(Exception):
            w.body_edits([bad])
    w.sync()


def test_gpu_edits_in_a_batch(gpu):
    """Edits addressed to world 1 of three identical worlds change world 1 only."""
    sc = scenes.pyramid(6)
    w = World([sc, sc, sc])
    for _ in range(10):
        w.step(DT, VI, PI)
    w.body_edits([(1, 4, "apply_linear_impulse", (5.0, 3.0, 0.0, 0.0), True),
                  (1, 7, "set_transform", (3.0, 9.0, 0.4), True)])
    for _ in range(10):
        w.step(DT, VI, PI)
    b0, b1, b2 = w.bodies(0), w.bodies(1), w.bodies(2)
    assert np.array_equal(b0, b2)
    assert not np.array_equal(b0, b1)
    with pytest.raises(Exception):
        w.body_edits([(3, 0, "set_awake", (1.0,), True)])
    w.sync()
