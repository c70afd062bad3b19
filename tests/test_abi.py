"""The C-ABI library loads, exports every symbol include/box2d_gb300.h declares, and its host-side
world setup (shape hulls, mass data, transforms, proxy ids, fat AABBs) equals the oracle's. None of
these calls touches a GPU."""
import os
import re

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes
from box2dpp_gb300.world import World

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "box2d_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:gb_status|const char\*|int)\s+(gb_\w+)\(", text, re.M)))


def test_header_matches_binding_list():
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert b"box2d_gb300" in lib.gb_version()


@pytest.mark.parametrize("make", [
    lambda: scenes.config1(),
    lambda: scenes.drop(300, scenes.SplitMix64(2)),
    lambda: scenes.chains(3, 6, scenes.SplitMix64(1)),
    lambda: scenes.stacks(50, scenes.SplitMix64(8)),
    lambda: scenes.chain_terrain(scenes.SplitMix64(12)),
])
def test_host_setup_equals_oracle(make):
    sc = make()
    g = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    assert np.array_equal(g.bodies().view(np.uint32), o.bodies().view(np.uint32))
    gi, gf = g.proxies()
    oi, of = o.proxies()
    assert np.array_equal(gi, oi)
    assert np.array_equal(gf.view(np.uint32), of.view(np.uint32))


def test_invalid_arguments_rejected():
    lib = _lib.load()
    import ctypes as C
    h = C.c_void_p()
    assert lib.gb_world_create(0, None, C.byref(h)) == _lib.GB_ERR_INVALID
    w = World(scenes.pyramid(2))
    bad = lib.gb_create_bodies(w.h, 5, 1, np.zeros(1, np.int32), np.zeros(9, np.float32),
                               np.zeros(1, np.int32), np.zeros(1, np.int32))
    assert bad == _lib.GB_ERR_INVALID
    bad = lib.gb_create_bodies(w.h, 0, 1, np.array([7], np.int32), np.zeros(9, np.float32),
                               np.zeros(1, np.int32), np.zeros(1, np.int32))
    assert bad == _lib.GB_ERR_INVALID


def test_joint_records_validated():
    """gb_create_joints refuses a gear joint that does not couple two existing revolute or prismatic
    joints (b2GearJoint.cpp:54-55 asserts the types), a gear index that is not an integer, and a
    pulley with ratio 0 (b2PulleyJoint.cpp:64); a valid gear is accepted."""
    lib = _lib.load()
    w = World(scenes.gears(scenes.SplitMix64(8)))
    out = np.zeros(1, np.int32)

    def joint(jtype, a, b, vals):
        f = np.zeros(12, np.float32)
        f[:len(vals)] = vals
        return lib.gb_create_joints(w.h, 0, 1, np.array([jtype], np.int32), np.array([a], np.int32),
                                    np.array([b], np.int32), f, np.zeros(1, np.int32), out)

    assert joint(scenes.GEAR, 1, 2, [0.0, 99.0, 1.0]) == _lib.GB_ERR_INVALID  # no joint 99
    assert joint(scenes.GEAR, 1, 2, [0.0, 2.0, 1.0]) == _lib.GB_ERR_INVALID   # joint 2 is a gear
    assert joint(scenes.GEAR, 1, 2, [0.5, 1.0, 1.0]) == _lib.GB_ERR_INVALID   # not an index
    assert joint(scenes.PULLEY, 1, 2, [0.0] * 10 + [0.0]) == _lib.GB_ERR_INVALID
    assert joint(11, 1, 2, []) == _lib.GB_ERR_INVALID
    n = len(scenes.gears(scenes.SplitMix64(8)).joints)
    assert joint(scenes.GEAR, 1, 2, [0.0, 1.0, 2.0]) == _lib.GB_OK and out[0] == n


def test_create_chain_matches_child_records():
    """gb_create_chain (b2ChainShape::CreateChain / CreateLoop + CreateFixture) makes the same child
    fixtures, proxies and fat AABBs as the scene's child-edge records, for an open chain with ghost
    vertices and a loop; too few vertices are refused."""
    import ctypes as C

    lib = _lib.load()
    pts = [(-6.0, 0.0), (-3.0, 1.0), (0.0, 0.5), (3.0, 1.5), (6.0, 0.0)]
    box = [(-2.0, -1.0), (2.0, -1.0), (2.0, 1.0), (-2.0, 1.0)]
    ref = scenes.Scene(name="chain_records")
    g = ref.body(scenes.STATIC, 0.0, 0.0)
    ref.chain(g, pts, prev=(-8.0, -1.0), next_=(8.0, -1.0), friction=0.5)
    k = ref.body(scenes.KINEMATIC, 1.0, 5.0, angle=0.3)
    ref.chain(k, box, loop=True, friction=0.5)
    want = World(ref)

    bare = scenes.Scene(name="chain_call")
    bare.body(scenes.STATIC, 0.0, 0.0)
    bare.body(scenes.KINEMATIC, 1.0, 5.0, angle=0.3)
    got = World(bare)
    mat = np.array([0.0, 0.5, 0.0], np.float32)
    filt = np.array([1, 0xFFFF, 0, 0], np.int32)
    first = C.c_int(-1)
    pn = np.array([-8.0, -1.0, 8.0, -1.0], np.float32)
    assert lib.gb_create_chain(got.h, 0, 0, np.array(pts, np.float32).ravel(), len(pts), 0, pn.ctypes.data, 3, mat,
                               filt, C.byref(first)) == _lib.GB_OK and first.value == 0
    assert lib.gb_create_chain(got.h, 0, 1, np.array(box, np.float32).ravel(), len(box), 1, None, 0, mat, filt,
                               C.byref(first)) == _lib.GB_OK and first.value == len(pts) - 1
    gi, gf = got.proxies()
    wi, wf = want.proxies()
    assert len(gi) == len(pts) - 1 + len(box)
    assert np.array_equal(gi, wi)
    assert np.array_equal(gf.view(np.uint32), wf.view(np.uint32))
    assert lib.gb_create_chain(got.h, 0, 1, np.array(box[:2], np.float32).ravel(), 2, 1, None, 0, mat, filt,
                               C.byref(first)) == _lib.GB_ERR_INVALID
