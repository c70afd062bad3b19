"""b2Body state changes between steps (SetTransform, SetLinearVelocity, SetAngularVelocity, SetAwake,
ApplyForce, ApplyForceToCenter, ApplyTorque, ApplyLinearImpulse, ApplyAngularImpulse, b2MouseJoint::SetTarget): the CPU
restatement against the compiled reference calling its own b2Body methods, bit for bit after every
step (project trig)."""
import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from tests._util import digest, edit_scene, edit_script, mouse_script


@pytest.mark.skipif(not oracle.reference_available(), reason="needs the reference source tree")
def test_port_edits_match_reference():
    sc = edit_scene()
    script = edit_script()
    ref = oracle.OracleWorld(sc, "reference", "project")
    port = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 341):
        for (op, body, vals, wake) in script.get(s, []):
            ref.body_edit(op, body, vals, wake)
            port.body_edit(op, body, vals, wake)
        ref.step()
        port.step()
        rb, pb = ref.bodies(), port.bodies()
        assert np.array_equal(rb.view(np.uint32), pb.view(np.uint32)), f"bodies differ at step {s}"
        ri, rf = ref.contacts()
        pi_, pf = port.contacts()
        assert np.array_equal(digest(rb, ri, rf), digest(pb, pi_, pf)), f"contacts differ at step {s}"
    # the script did something: the kinematic paddle was moved, a sleeping body stayed asleep
    assert pb[56, 0] != sc.bodies[56][1][0]


@pytest.mark.skipif(not oracle.reference_available(), reason="needs the reference source tree")
def test_port_mouse_targets_match_reference():
    """b2MouseJoint::SetTarget between steps (dragging, a force-bounded joint, waking a sleeping body)
    on the pulley and mouse joint scene, bit for bit against the reference every step."""
    sc = scenes.pulley_mouse(scenes.SplitMix64(4))
    script = mouse_script()
    ref = oracle.OracleWorld(sc, "reference", "project")
    port = oracle.OracleWorld(sc, "port", "project")
    asleep_before_target = False
    for s in range(1, 361):
        for (op, body, vals, wake) in script.get(s, []):
            if s == 331:
                asleep_before_target = port.bodies()[7, 11] == 0.0
            ref.body_edit(op, body, vals, wake)
            port.body_edit(op, body, vals, wake)
        ref.step()
        port.step()
        rb, pb = ref.bodies(), port.bodies()
        assert np.array_equal(rb.view(np.uint32), pb.view(np.uint32)), f"bodies differ at step {s}"
        ri, rf = ref.contacts()
        pi_, pf = port.contacts()
        assert np.array_equal(digest(rb, ri, rf), digest(pb, pi_, pf)), f"contacts differ at step {s}"
    assert asleep_before_target and pb[7, 11] == 1.0
    # the dragged box followed its last target
    assert abs(pb[6, 0] - 13.94) < 0.2 and abs(pb[6, 1] - 3.35) < 0.2
