"""The C++ mirror of b2World (include/box2d_gb300.hpp) builds against the library and, on the GPU,
runs the Box2D manual's HelloWorld bit for bit like the CPU oracle."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SRC = os.path.join(ROOT, "tests", "cpp", "hello_world.cpp")


def _compile(tmp_path):
    lib = _lib.library_path()
    if not os.path.exists(lib):
        from box2dpp_gb300 import build
        build.build()
    exe = str(tmp_path / "hello_world")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_mirror_compiles_and_links(tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
def test_hello_world_matches_oracle(gpu, tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    got = np.array([[float.fromhex(v) for v in ln.split()[1:]] for ln in lines[:60]], dtype=np.float32)
    sc = scenes.Scene(name="hello_world")
    g = sc.body(scenes.STATIC, 0.0, -10.0)
    sc.fixture(g, 3, [50.0, 10.0], n=2, density=0.0)
    b = sc.body(scenes.DYNAMIC, 0.0, 4.0)
    sc.fixture(b, 3, [1.0, 1.0], n=2, density=1.0, friction=0.3)
    o = oracle.OracleWorld(sc, "port", "project")
    o.record_events(True)
    want = []
    kinds = np.zeros(4, dtype=np.int64)
    last_post = None
    for _ in range(60):
        o.step(1.0 / 60.0, 6, 2)
        s = o.bodies()[1]
        want.append([s[0], s[1], s[2]])
        ev, imp = o.events()
        for k, row in zip(ev[:, 0], imp):
            kinds[k] += 1
            if k == 3:
                last_post = row[0]
    want = np.array(want, dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the listener saw the reference's calls: counts per kind and the last PostSolve impulse
    tail = lines[60].split()
    assert tail[0] == "contacts" and int(tail[1]) == 1
    assert [int(tail[3]), int(tail[5]), int(tail[9]), int(tail[11])] == [kinds[0], kinds[1], kinds[2], kinds[3]]
    assert kinds[3] > 0
    assert np.float32(float.fromhex(tail[13])).view(np.uint32) == np.float32(last_post).view(np.uint32)


EDITS_SRC = os.path.join(ROOT, "tests", "cpp", "body_edits.cpp")


def _compile_edits(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "body_edits")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), EDITS_SRC, "-o",
           exe, "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_body_edits_compile(tmp_path):
    _compile_edits(tmp_path)


@pytest.mark.gpu
def test_cpp_body_edits_match_oracle(gpu, tmp_path):
    """b2Body::ApplyLinearImpulse, SetTransform, SetAngularVelocity, ApplyForce, ApplyTorque,
    SetLinearVelocity and SetAwake through the C++ mirror, bit for bit like the CPU oracle."""
    from tests._util import (APPLY_FORCE, APPLY_LINEAR_IMPULSE, APPLY_TORQUE, SET_ANGULAR_VELOCITY, SET_AWAKE,
                             SET_LINEAR_VELOCITY, SET_TRANSFORM)

    exe = _compile_edits(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.array([[float.fromhex(v) for v in ln.split()[1:4]] for ln in r.stdout.strip().splitlines()],
                   dtype=np.float32)
    sc = scenes.Scene(name="body_edits")
    g = sc.body(scenes.STATIC, 0.0, -10.0)
    sc.fixture(g, 3, [50.0, 10.0], n=2, density=0.0)
    b = sc.body(scenes.DYNAMIC, 0.0, 4.0)
    sc.fixture(b, 3, [1.0, 1.0], n=2, density=1.0, friction=0.3)
    o = oracle.OracleWorld(sc, "port", "project")
    script = {10: (APPLY_LINEAR_IMPULSE, (3.0, 6.0, 0.5, 3.0)), 25: (SET_TRANSFORM, (-4.0, 6.0, 0.6)),
              30: (SET_ANGULAR_VELOCITY, (3.0,)), 40: (APPLY_FORCE, (50.0, 0.0, -4.0, 1.0)),
              41: (APPLY_TORQUE, (-20.0,)), 60: (SET_LINEAR_VELOCITY, (1.0, 0.0)), 75: (SET_AWAKE, (0.0,))}
    want = []
    for i in range(90):
        if i in script:
            op, vals = script[i]
            o.body_edit(op, 1, vals, True)
        o.step(1.0 / 60.0, 8, 3)
        s = o.bodies()[1]
        want.append([s[0], s[1], s[2]])
    want = np.array(want, dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


MOUSE_PULLEY_SRC = os.path.join(ROOT, "tests", "cpp", "mouse_pulley.cpp")


def _compile_mouse_pulley(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "mouse_pulley")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), MOUSE_PULLEY_SRC,
           "-o", exe, "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_mouse_pulley_compile(tmp_path):
    _compile_mouse_pulley(tmp_path)


@pytest.mark.gpu
def test_cpp_mouse_pulley_match_oracle(gpu, tmp_path):
    """b2PulleyJointDef::Initialize and b2MouseJoint::SetTarget through the C++ mirror, bit for bit
    like the CPU oracle on the same scene (the pulley's anchors and lengths are exact in float)."""
    from tests._util import MOUSE_TARGET

    exe = _compile_mouse_pulley(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.array([[float.fromhex(v) for v in ln.split()[1:]] for ln in r.stdout.strip().splitlines()],
                   dtype=np.float32)
    sc = scenes.Scene(name="mouse_pulley")
    g = sc.body(scenes.STATIC, 0.0, -10.0)
    sc.fixture(g, 3, [50.0, 10.0], n=2, density=0.0)
    anchor = sc.body(scenes.STATIC, 0.0, 0.0)
    a = sc.body(scenes.DYNAMIC, -3.0, 5.0)
    sc.fixture(a, 3, [0.5, 1.0], n=2, density=1.0)
    b = sc.body(scenes.DYNAMIC, 3.0, 4.0)
    sc.fixture(b, 3, [0.5, 1.0], n=2, density=1.0)
    sc.pulley(a, b, (-3.0, 10.0), (3.0, 10.0), (0.0, 1.0), (0.0, 1.0), 4.0, 5.0, 1.2)
    d = sc.body(scenes.DYNAMIC, 0.0, 3.0)
    sc.fixture(d, 3, [0.5, 0.5], n=2, density=1.0)
    sc.mouse(anchor, d, (0.25, 3.25), 200.0)
    o = oracle.OracleWorld(sc, "port", "project")
    want = []
    for i in range(120):
        if 10 <= i < 70:
            o.body_edit(MOUSE_TARGET, 1, (0.25 + 0.125 * (i - 10), 3.25), True)
        o.step(1.0 / 60.0, 8, 3)
        s = o.bodies()
        want.append([s[k, c] for k in (a, b, d) for c in (0, 1, 2)])
    want = np.array(want, dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the dragged box followed the target to the right, the pulley moved
    assert want[-1, 6] > 5.0 and want[-1, 1] != 5.0


CHAIN_SRC = os.path.join(ROOT, "tests", "cpp", "chain.cpp")


def _compile_chain(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "chain")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), CHAIN_SRC, "-o", exe,
           "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_chain_compile(tmp_path):
    _compile_chain(tmp_path)


def chain_scene():
    """The scene tests/cpp/chain.cpp builds, as scene records."""
    sc = scenes.Scene(name="chain_cpp")
    g = sc.body(scenes.STATIC, 0.0, 0.0)
    terrain = [(-8.0 + 2.0 * i, 0.5 if i % 2 else 0.0) for i in range(9)]
    sc.chain(g, terrain, prev=(-10.0, 1.0), next_=(10.0, 1.0), friction=0.6)
    c = sc.body(scenes.STATIC, 14.0, 4.0, angle=0.2)
    sc.chain(c, [(-3.0, -2.0), (3.0, -2.0), (3.0, 2.0), (-3.0, 2.0)], loop=True, friction=0.4)
    for i in range(8):
        b = sc.body(scenes.DYNAMIC, -7.0 + 2.5 * i if i < 6 else 13.0 + 2.0 * (i - 6), 3.0 if i < 6 else 4.0,
                    angle=float(np.float32(0.1) * np.float32(i)))
        if i % 2:
            sc.fixture(b, scenes.CIRCLE, [0.0, 0.0, 0.4], 1, density=1.0, friction=0.4)
        else:
            sc.fixture(b, scenes.BOX, [0.4, 0.3], 2, density=1.0, friction=0.4)
    return sc


@pytest.mark.gpu
def test_cpp_chain_match_oracle(gpu, tmp_path):
    """b2ChainShape::CreateChain / CreateLoop through the C++ mirror: positions bit for bit like the
    CPU oracle (itself bit-exact with the reference's b2ChainShape), and the contacts' chain child
    indices (b2Contact::GetChildIndexA) as the oracle's fixture ids give them."""
    exe = _compile_chain(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    got = np.array([[float.fromhex(v) for v in ln.split()[1:]] for ln in lines[:120]], dtype=np.float32)
    got_children = sorted(tuple(int(t) for t in ln.split()[1::2]) for ln in lines[120:])
    sc = chain_scene()
    o = oracle.OracleWorld(sc, "port", "project")
    want = []
    for _ in range(120):
        o.step(1.0 / 60.0, 8, 3)
        s = o.bodies()
        want.append([s[k, c] for k in range(2, 10) for c in (0, 1)])
    want = np.array(want, dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    ci, _ = o.contacts()
    fbody = [f[0] for f in sc.fixtures]
    want_children = sorted((0 if f < 8 else 1, f if f < 8 else f - 8, fbody[fb]) for f, fb in zip(ci[:, 0], ci[:, 1])
                           if f < 12)
    assert got_children == want_children and len(want_children) > 0
