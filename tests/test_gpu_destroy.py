"""Destruction between device steps: b2World::DestroyBody / DestroyJoint and b2Body::DestroyFixture,
with bodies created afterwards, bit-exact against the reference's golden digests step by step, with
the reference's destruction-listener calls and proxy ids; EndContact calls as the CPU oracle makes
them; and a batch where one world changes while the others step on."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, apply_ops, destroy_script, digest, golden

pytestmark = pytest.mark.gpu


def test_destroy_case_bit_exact_vs_reference(gpu):
    g = golden("destroy_mix_project")
    w = World(scenes.destroy_mix(scenes.SplitMix64(5)))
    script = destroy_script()
    calls = []
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            calls += [(s, k, i) for (k, i) in apply_ops(w, script[s])]
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    w.sync()
    assert np.array_equal(np.array(calls, np.int32).reshape(-1, 3), g["goodbyes"])
    ids, _ = w.proxies()
    assert np.array_equal(ids, g["proxy_ids"])


def test_destroy_end_contact_calls_match_oracle(gpu):
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    o.record_events(True)
    script = destroy_script()
    ended = 0
    for s in range(1, 161):
        if s in script:
            before = len(o.events()[0])
            for op in script[s]:
                if op[0] == "add":
                    apply_ops(w, [op])
                    apply_ops(o, [op])
                    continue
                got = getattr(w, "destroy_" + op[0])(op[1])
                getattr(o, "destroy_" + op[0])(op[1])
                ev, _ = o.events()
                mine = got[got[:, 0] == 2][:, 1:]
                theirs = ev[before:][ev[before:, 0] == 1][:, 1:]
                assert np.array_equal(mine, theirs), (s, op, mine, theirs)
                ended += len(mine)
                before = len(ev)
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
    assert ended > 0


def test_destroy_in_one_world_of_a_batch(gpu):
    scs = [scenes.pyramid(6), scenes.destroy_mix(scenes.SplitMix64(5)), scenes.drop(120, scenes.SplitMix64(3))]
    w = World(scs)
    os_ = [oracle.OracleWorld(sc, "port", "project") for sc in scs]
    script = destroy_script()
    for s in range(1, 121):
        if s in script:
            assert apply_ops(w, script[s], w=1) == apply_ops(os_[1], script[s])
        w.step(DT, VI, PI)
        for o in os_:
            o.step(DT, VI, PI)
        if s % 20 == 0:
            for i, o in enumerate(os_):
                assert np.array_equal(w.bodies(i).view(np.uint32), o.bodies().view(np.uint32)), (s, i)
                gi, gf = w.contacts(i)
                oi, of = o.contacts()
                assert np.array_equal(gi, oi) and np.array_equal(gf.view(np.uint32), of.view(np.uint32)), (s, i)
