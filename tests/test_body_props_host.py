"""b2Body property changes on the host before any step (no GPU needed): mass data set and reset, type,
fixed rotation, bullet, sleeping, damping and gravity scale, read back through gb_get_body_info and
compared with the reference's b2Body getters (the restatement on hosts without the reference tree)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300._lib import (BODY_BULLET, BODY_FIXED_ROTATION, BODY_GRAVITY_SCALE, BODY_LINEAR_DAMPING,
                                BODY_MASS_DATA, BODY_RESET_MASS_DATA, BODY_SLEEPING_ALLOWED, BODY_TYPE, GbError)
from box2dpp_gb300.world import World

OPS = [(47, BODY_MASS_DATA, (3.0, 0.2, -0.1, 2.5)), (13, BODY_MASS_DATA, (0.5, 0.0, 0.0, 0.0)),
       (14, BODY_MASS_DATA, (-1.0, 0.3, 0.3, 4.0)),        # mass <= 0 becomes 1
       (37, BODY_MASS_DATA, (5.0, 0.0, 0.0, 1.0)),         # a static body keeps its mass data
       (15, BODY_FIXED_ROTATION, 1.0), (15, BODY_MASS_DATA, (2.0, 0.1, 0.0, 3.0)),  # no inertia
       (16, BODY_BULLET, 1.0), (17, BODY_SLEEPING_ALLOWED, 0.0), (18, BODY_LINEAR_DAMPING, 0.7),
       (19, BODY_GRAVITY_SCALE, -2.0), (20, BODY_TYPE, 1.0), (47, BODY_RESET_MASS_DATA, 0.0)]


def test_body_info_after_host_changes_matches():
    sc = scenes.destroy_mix(scenes.SplitMix64(11))
    w = World(sc)
    o = oracle.OracleWorld(sc, "reference" if oracle.reference_available() else "port", "project")
    for i, (body, prop, v) in enumerate(OPS):
        w.body_set(body, prop, v)
        o.body_set(body, prop, v)
        for b in range(len(sc.bodies)):
            (a, fa), (c, fc) = w.body_info(b), o.body_info(b)
            assert fa == fc and np.array_equal(a.view(np.uint32), c.view(np.uint32)), (i, b, a, c)
    # the moved centre of mass shows in the body state (world centre, velocity) too
    assert np.array_equal(w.bodies().view(np.uint32), o.bodies().view(np.uint32))


def test_body_info_rejects_bad_bodies():
    w = World(scenes.pyramid(3))
    with pytest.raises(GbError):
        w.body_info(1000)
    with pytest.raises(GbError):
        w.body_set(0, 10, 0.0)


def test_fixture_queries_before_stepping_match_reference():
    """b2Fixture::TestPoint, RayCast, GetAABB and GetMassData on the host copy (no step yet) against the
    reference's for seeded points and rays around every fixture."""
    if not oracle.reference_available():
        pytest.skip("reference tree not present")
    import importlib.util
    import os

    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    w = World(sc)
    r = oracle.OracleWorld(sc, "reference", "project")
    for q in mod.fixture_query_inputs(r.bodies(), sc.arrays()["fix_body"], seed=11):
        a, b = w.fixture_query(int(q[0]), int(q[1]), q[2:]), r.fixture_query(int(q[0]), int(q[1]), q[2:])
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (q, a, b)
    # b2Fixture::GetMassData of every fixture (op 3)
    for f in range(len(sc.fixtures)):
        a, b = w.fixture_query(f, 3), r.fixture_query(f, 3)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (f, a, b)
