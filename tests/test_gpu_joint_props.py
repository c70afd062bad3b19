"""Joint setters between device steps (gb_joint_set: motor speed, torque and force, motor and limit
switches, limits, the distance joint's length, springs, rope length, friction and motor-joint forces,
offsets and correction): bit-exact against the reference's golden digests step by step on a car,
rope, friction and motor scene, a prismatic scene and a distance and weld scene; properties a joint
type does not have are refused."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300._lib import GbError
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, apply_ops, digest, golden, joint_scripts

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["joint_props_zoo", "joint_props_prismatic", "joint_props_mix"])
def test_joint_props_bit_exact_vs_reference(gpu, case):
    make, _, script = joint_scripts()[case]
    g = golden(f"{case}_project")
    w = World(make())
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(w, script[s])
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"


def test_joint_set_rejects_what_a_type_does_not_have(gpu):
    w = World(scenes.joint_zoo(scenes.SplitMix64(6)))  # 0 wheel, 2 rope, 7 friction, 10 motor
    for joint, prop in [(0, 3), (0, 4), (2, 0), (7, 5), (10, 14), (0, 15)]:
        with pytest.raises(GbError):
            w.joint_set(joint, prop, 1.0)
    with pytest.raises(GbError):
        w.joint_set(99, 0, 1.0)
    w2 = World(scenes.prismatic_mix(scenes.SplitMix64(5)))
    with pytest.raises(GbError):
        w2.joint_set(0, 4, (1.0, -1.0))  # lower above upper


@pytest.mark.parametrize("name,seed", [("joint_zoo", 6), ("prismatic_mix", 5), ("joint_mix", 3), ("pulley_mouse", 4),
                                       ("gears", 8)])
def test_joint_reactions_match_oracle(gpu, name, seed):
    """b2Joint::GetReactionForce / GetReactionTorque of every joint after 50 device steps, against the
    CPU restatement (itself bit-exact with the reference)."""
    import oracle

    sc = getattr(scenes, name)(scenes.SplitMix64(seed))
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for _ in range(50):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    for j in range(len(sc.joints)):
        a, b = w.joint_reaction(j, 60.0), o.joint_reaction(j, 60.0)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (j, a, b)
