"""b2Body state changes between steps (SetTransform, SetLinearVelocity, SetAngularVelocity, SetAwake,
ApplyForce, ApplyForceToCenter, ApplyTorque, ApplyLinearImpulse, ApplyAngularImpulse): the CPU
restatement against the compiled reference calling its own b2Body methods, bit for bit after every
step (project trig)."""
import numpy as np
import pytest

import oracle
from tests._util import digest, edit_scene, edit_script


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
