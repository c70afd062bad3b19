"""b2Body properties changed between device steps (SetType to static, kinematic and dynamic, SetActive
off and on, SetFixedRotation, SetBullet, SetSleepingAllowed, SetLinearDamping, SetAngularDamping,
SetGravityScale, SetMassData, ResetMassData) and fixture properties (SetSensor, SetFriction,
SetRestitution, SetFilterData, SetDensity) and b2World::ShiftOrigin: bit-exact against the reference's golden digests step by step with the reference's
final proxy ids; the EndContact calls of the contacts SetType and SetActive destroy as the CPU oracle
makes them; and one world of a batch changed while the others step on."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300._lib import GbError
from box2dpp_gb300.world import World
from tests._util import (DT, PI, VI, apply_ops, body_props_script, digest, fixture_props_script, golden,
                         shift_script)

pytestmark = pytest.mark.gpu


def test_body_props_case_bit_exact_vs_reference(gpu):
    g = golden("body_props_project")
    w = World(scenes.destroy_mix(scenes.SplitMix64(11)))
    script = body_props_script()
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(w, script[s])
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    w.sync()
    ids, _ = w.proxies()
    assert np.array_equal(ids, g["proxy_ids"])
    # mass data, damping and flags as the CPU restatement has them after the same script
    o = oracle.OracleWorld(scenes.destroy_mix(scenes.SplitMix64(11)), "port", "project")
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(o, script[s])
        o.step(DT, VI, PI)
    for b in range(w.n_bodies[0]):
        (a, fa), (c, fc) = w.body_info(b), o.body_info(b)
        assert fa == fc and np.array_equal(a.view(np.uint32), c.view(np.uint32)), (b, a, c)


def test_fixture_props_case_bit_exact_vs_reference(gpu):
    g = golden("fixture_props_project")
    w = World(scenes.destroy_mix(scenes.SplitMix64(13)))
    script = fixture_props_script()
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(w, script[s])
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    w.sync()
    ids, _ = w.proxies()
    assert np.array_equal(ids, g["proxy_ids"])


def test_shift_origin_case_bit_exact_vs_reference(gpu):
    g = golden("shift_origin_project")
    w = World(scenes.pulley_mouse(scenes.SplitMix64(4)))
    script = shift_script()
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(w, script[s])
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    w.sync()
    ids, fat = w.proxies()
    assert np.array_equal(ids, g["proxy_ids"])
    assert np.array_equal(fat.view(np.uint32), g["proxy_fat"].view(np.uint32))


def test_body_props_end_contact_calls_match_oracle(gpu):
    sc = scenes.destroy_mix(scenes.SplitMix64(11))
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    o.record_events(True)
    script = body_props_script()
    ended = 0
    for s in range(1, 221):
        for op in script.get(s, []):
            before = len(o.events()[0])
            got = w.body_set(op[1], op[2], op[3])
            o.body_set(op[1], op[2], op[3])
            ev, _ = o.events()
            theirs = ev[before:][ev[before:, 0] == 1][:, 1:]
            assert np.array_equal(got[:, 1:], theirs), (s, op, got, theirs)
            assert np.all(got[:, 0] == 2)
            ended += len(got)
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    assert ended > 0


def test_body_props_in_one_world_of_a_batch(gpu):
    scs = [scenes.pyramid(6), scenes.destroy_mix(scenes.SplitMix64(11)), scenes.drop(120, scenes.SplitMix64(3))]
    alone = World([scs[0], scs[1]])
    batch = World(scs)
    script = body_props_script()
    for s in range(1, 221):
        if s in script:
            apply_ops(batch, script[s], w=1)
            apply_ops(alone, script[s], w=1)
        batch.step(DT, VI, PI)
        alone.step(DT, VI, PI)
    batch.sync()
    alone.sync()
    # world 0 is untouched by world 1's changes, and world 1 steps as it does beside one world only
    for k in (0, 1):
        assert np.array_equal(batch.bodies(k).view(np.uint32), alone.bodies(k).view(np.uint32)), k


def test_body_set_rejects_bad_arguments(gpu):
    w = World(scenes.pyramid(3))
    with pytest.raises(GbError):
        w.body_set(0, 10, 1.0)
    with pytest.raises(GbError):
        w.body_set(0, 0, 5.0)
    with pytest.raises(GbError):
        w.body_set(10_000, 3, 1.0)
    with pytest.raises(GbError):
        w.fixture_set(1, 5, 0.0)
    with pytest.raises(GbError):
        w.fixture_set(1, 2, -1.0)  # negative density
