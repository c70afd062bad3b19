"""The C++ mirror of b2World (include/box2d_gb300.hpp) builds against the library and, on the GPU,
runs the Box2D manual's HelloWorld bit for bit like the CPU oracle."""
from __future__ import annotations

import ctypes as C
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


DQ_SRC = os.path.join(ROOT, "tests", "cpp", "destroy_queries.cpp")


def _compile_dq(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "destroy_queries")
    libdir = os.path.dirname(lib)
    # without contraction: GetWorldManifold runs in the caller's code and is compared bit for bit
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           DQ_SRC, "-o", exe, "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _dq_scene():
    s = scenes.Scene(name="destroy_queries")
    g = s.body(scenes.STATIC, 0.0, 0.0)
    s.fixture(g, scenes.EDGE, [-20.0, 0.0, 20.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    for r in range(3):
        for j in range(4 - r):
            b = s.body(scenes.DYNAMIC, float(np.float32(-1.875 + r * 0.625 + j * 1.25)), 0.5 + r * 1.0)
            s.fixture(b, scenes.BOX, [0.5, 0.5], 2, density=5.0, friction=0.6)
    a = s.body(scenes.STATIC, 6.0, 6.0)
    s.fixture(a, scenes.CIRCLE, [0.0, 0.0, 0.25])
    bob = s.body(scenes.DYNAMIC, 8.0, 6.0)
    s.fixture(bob, scenes.CIRCLE, [0.0, 0.0, 0.5], density=1.0)
    s.revolute(a, bob, [0.0, 0.0], [-2.0, 0.0])
    t = s.body(scenes.DYNAMIC, -6.0, 3.0)
    s.fixture(t, scenes.BOX, [0.5, 0.25], 2, density=1.0)
    s.fixture(t, scenes.CIRCLE, [0.5, 0.0, 0.25], density=2.0)
    return s


def _world_manifold(m_ints, m_flts, xa, ra, xb, rb):
    """b2WorldManifold::Initialize (b2Collision.cpp:25-66) in float32, operation for operation."""
    f = np.float32
    mul = lambda x, v: (f(f(x[3] * v[0]) - f(x[2] * v[1])) + x[0], f(f(x[2] * v[0]) + f(x[3] * v[1])) + x[1])
    rot = lambda x, v: (f(x[3] * v[0]) - f(x[2] * v[1]), f(x[2] * v[0]) + f(x[3] * v[1]))
    dot = lambda a, b: f(a[0] * b[0]) + f(a[1] * b[1])
    kind, count = int(m_ints[4]), int(m_ints[3])
    assert count > 0  # Initialize returns at once for an empty manifold
    ln, lp = (m_flts[0], m_flts[1]), (m_flts[2], m_flts[3])
    pts = [(m_flts[4], m_flts[5]), (m_flts[8], m_flts[9])]
    pts_out, seps = [(f(0), f(0)), (f(0), f(0))], [f(0), f(0)]
    if kind == 0:
        normal = (f(1), f(0))
        pa, pb = mul(xa, lp), mul(xb, pts[0])
        d = (pa[0] - pb[0], pa[1] - pb[1])
        eps = f(np.finfo(np.float32).eps)
        if dot(d, d) > f(eps * eps):
            normal = (pb[0] - pa[0], pb[1] - pa[1])
            length = np.sqrt(f(f(normal[0] * normal[0]) + f(normal[1] * normal[1])), dtype=np.float32)
            if length >= eps:
                inv = f(f(1) / length)
                normal = (f(normal[0] * inv), f(normal[1] * inv))
        ca = (pa[0] + f(ra * normal[0]), pa[1] + f(ra * normal[1]))
        cb = (pb[0] - f(rb * normal[0]), pb[1] - f(rb * normal[1]))
        pts_out[0] = (f(f(0.5) * f(ca[0] + cb[0])), f(f(0.5) * f(ca[1] + cb[1])))
        seps[0] = dot((cb[0] - ca[0], cb[1] - ca[1]), normal)
    else:
        xp, xq = (xa, xb) if kind == 1 else (xb, xa)
        rp, rq = (ra, rb) if kind == 1 else (rb, ra)
        normal = rot(xp, ln)
        plane = mul(xp, lp)
        for i in range(count):
            clip = mul(xq, pts[i])
            s = f(rp - dot((clip[0] - plane[0], clip[1] - plane[1]), normal))
            cp_ = (clip[0] + f(s * normal[0]), clip[1] + f(s * normal[1]))
            cq = (clip[0] - f(rq * normal[0]), clip[1] - f(rq * normal[1]))
            ca, cb = (cp_, cq) if kind == 1 else (cq, cp_)
            pts_out[i] = (f(f(0.5) * f(ca[0] + cb[0])), f(f(0.5) * f(ca[1] + cb[1])))
            seps[i] = dot((cb[0] - ca[0], cb[1] - ca[1]), normal) if kind == 1 else \
                dot((ca[0] - cb[0], ca[1] - cb[1]), normal)
        if kind == 2:
            normal = (-normal[0], -normal[1])
    return np.array([normal[0], normal[1], pts_out[0][0], pts_out[0][1], pts_out[1][0], pts_out[1][1], seps[0],
                     seps[1]], dtype=np.float32)


@pytest.mark.gpu
def test_cpp_destroy_queries_match_oracle(gpu, tmp_path):
    """DestroyBody / DestroyFixture / SetDestructionListener, GetBodyList, GetProxyCount, QueryAABB and
    RayCast callbacks and GetWorldManifold of the C++ mirror against the CPU oracle (state, listener
    calls, proxies, manifold bits) and against the device queries (callback protocol)."""
    from box2dpp_gb300.world import World

    exe = _compile_dq(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = {}
    bodies = {}
    for ln in r.stdout.strip().splitlines():
        parts = ln.split()
        if parts[0] == "body":
            bodies[int(parts[1])] = np.array([float.fromhex(v) for v in parts[2:]], dtype=np.float32)
        else:
            out[parts[0]] = parts[1:]
    sc = _dq_scene()
    o = oracle.OracleWorld(sc, "port", "project")
    o.record_events(True)
    gw = World(sc)
    ends, goodbyes = 0, []

    def step(n):
        nonlocal ends
        for _ in range(n):
            o.step(1.0 / 60.0, 8, 3)
            gw.step(1.0 / 60.0, 8, 3)
            ends += int((o.events()[0][:, 0] == 1).sum())

    def destroy(kind, i):
        nonlocal ends
        seen = len(o.events()[0])
        goodbyes.extend(int(x) for row in getattr(o, "destroy_" + kind)(i) for x in row)
        getattr(gw, "destroy_" + kind)(i)
        ends += int((o.events()[0][seen:, 0] == 1).sum())

    step(40)
    destroy("body", 5)
    destroy("fixture", 13)
    assert int(out["ends_after_first"][0]) == ends
    step(20)
    destroy("body", 10)
    for w_ in (o, gw):
        b = w_.add_body(2, [0.0, 8.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0], 1 | 2 | 16)
        w_.add_fixture(b, 3, [0.5, 0.5], 2, [1.0, 0.2, 0.0], [1, 0xFFFF, 0, 0])
    step(40)
    assert [int(x) for x in out["goodbyes"]] == goodbyes
    e = out["ends"]
    assert int(e[0]) == ends
    ob = o.bodies()
    alive = [i for i in range(len(ob)) if i not in (5, 10)]
    assert int(e[2]) == len(alive) and int(e[4]) == 0
    ids, _ = o.proxies()
    assert int(e[6]) == int((ids >= 0).sum())
    assert [int(x) for x in out["list"]] == sorted(alive, reverse=True)
    for i, got in bodies.items():
        want = ob[i][[0, 1, 2, 5, 6, 7]]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i
    q = gw.query_aabb(np.array([[-3.0, -1.0, 3.0, 2.0]], np.float32))[0]
    assert [int(x) for x in out["query"]] == list(q)
    assert [int(x) for x in out["query_stop"]] == list(q[:2])
    ray = np.array([-10.0, 0.75, 10.0, 0.25], np.float32)
    fix, hit = gw.raycast(ray[None, :])
    allf, _ = gw.raycast_all(ray)
    rr = out["ray"]
    assert int(rr[0]) == int(fix[0]) and int(rr[-1]) == len(allf)
    got = np.array([float.fromhex(v) for v in rr[1:6]], dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), hit[0].view(np.uint32))
    # contact edges per body: the device's contacts that involve the body
    fb = {f: b for f, b in enumerate(sc.arrays()["fix_body"])}
    fb[14] = 13  # the body created after the destructions
    gci, _ = gw.contacts()
    for item in out["edges"]:
        b, n = (int(x) for x in item.split(":"))
        want = sum(1 for row in gci if fb[int(row[0])] == b or fb[int(row[1])] == b)
        assert n == want, (b, n, want)
    fq = out["fixq"]
    bob = gw.bodies()[11]
    cx, cy = np.float32(bob[0]), np.float32(bob[1])
    ray = gw.fixture_query(11, 1, (cx - np.float32(2.0), cy + np.float32(0.1), cx + np.float32(2.0), cy - np.float32(0.1), 1.0))
    box = gw.fixture_query(11, 2)
    assert int(fq[0]) == int(gw.fixture_query(11, 0, (cx, cy))[0]) == 1
    assert int(fq[1]) == int(ray[0]) == 1
    got = np.array([float.fromhex(v) for v in fq[2:]], dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), np.concatenate([ray[1:], box]).view(np.uint32))
    th, tb, tq = o.tree_stats()
    t = out["tree"]
    assert [int(t[0]), int(t[1])] == [th, tb]
    assert np.float32(float.fromhex(t[2])).view(np.uint32) == tq.view(np.uint32)
    ci, cf = o.contacts()
    m = out["manifold"]
    k = int(m[0])
    assert k == int(np.argmax(ci[:, 3] > 0))
    ci, cf, m = ci[k:], cf[k:], m[1:]
    assert [int(m[0]), int(m[1]), int(m[2])] == [int(ci[0, 0]), int(ci[0, 1]), int(ci[0, 3])]
    fx_body = {f: b for f, b in enumerate(sc.arrays()["fix_body"])}
    fx_body[14] = 13  # the body created after the destructions
    radius = lambda f: (np.float32(sc.fixtures[f][2][2]) if f < len(sc.fixtures) and sc.fixtures[f][1] == scenes.CIRCLE
                        else np.float32(0.01))
    xf = lambda b: np.array([ob[b][0], ob[b][1], ob[b][8], ob[b][9]], dtype=np.float32)
    want = _world_manifold(ci[0], cf[0], xf(fx_body[int(ci[0, 0])]), radius(int(ci[0, 0])), xf(fx_body[int(ci[0, 1])]),
                           radius(int(ci[0, 1])))
    got = np.array([float.fromhex(v) for v in m[3:]], dtype=np.float32)
    n = int(ci[0, 3])
    sel = [0, 1] + [2 + 2 * k for k in range(n)] + [3 + 2 * k for k in range(n)] + [6 + k for k in range(n)]
    assert np.array_equal(got[sel].view(np.uint32), want[sel].view(np.uint32)), (got, want)
    assert int(out["profile"][0]) == 1


BP_SRC = os.path.join(ROOT, "tests", "cpp", "body_props.cpp")


def _compile_bp(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "body_props")
    libdir = os.path.dirname(lib)
    # without contraction: the frame getters run in the caller's code and are compared bit for bit
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           BP_SRC, "-o", exe,
           "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_body_props_compile(tmp_path):
    _compile_bp(tmp_path)


@pytest.mark.gpu
def test_cpp_body_props_match_oracle(gpu, tmp_path):
    """b2Body::SetType, SetActive, SetFixedRotation, SetBullet, SetSleepingAllowed, SetLinearDamping,
    SetAngularDamping and SetGravityScale of the C++ mirror against the CPU oracle: body states bit
    for bit and the contact listener's EndContact count (the ones the changes make included)."""
    exe = _compile_bp(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out, bodies = {}, {}
    for ln in r.stdout.strip().splitlines():
        parts = ln.split()
        if parts[0] == "body":
            bodies[int(parts[1])] = np.array([float.fromhex(v) for v in parts[2:]], dtype=np.float32)
        else:
            out[parts[0]] = parts[1:]
    o = oracle.OracleWorld(_dq_scene(), "port", "project")
    o.record_events(True)
    ends = 0

    def step(n):
        nonlocal ends
        for _ in range(n):
            o.step(1.0 / 60.0, 8, 3)
            ends += int((o.events()[0][:, 0] == 1).sum())

    def prop(body, p, v):
        nonlocal ends
        seen = len(o.events()[0])
        o.body_set(body, p, v)
        ends += int((o.events()[0][seen:, 0] == 1).sum())

    step(40)
    prop(2, _lib.BODY_TYPE, 0.0)
    prop(8, _lib.BODY_ACTIVE, 0.0)
    prop(11, _lib.BODY_GRAVITY_SCALE, 0.5)
    prop(11, _lib.BODY_LINEAR_DAMPING, 0.5)
    o.fixture_set(4, _lib.FIXTURE_FRICTION, 0.0)
    o.fixture_set(3, _lib.FIXTURE_RESTITUTION, 0.5)
    o.fixture_set(7, _lib.FIXTURE_SENSOR, 1.0)
    o.fixture_set(8, _lib.FIXTURE_FILTER, (1.0, 0xFFFF, -3.0))
    o.fixture_set(9, _lib.FIXTURE_FILTER, (1.0, 0xFFFF, -3.0))
    first = out["ends_after_first"]  # "<count> type <type of the box>"
    assert [int(first[0]), int(first[2])] == [ends, 0]
    step(20)
    prop(8, _lib.BODY_ACTIVE, 1.0)
    prop(2, _lib.BODY_TYPE, 2.0)
    o.fixture_set(7, _lib.FIXTURE_SENSOR, 0.0)
    o.fixture_set(9, _lib.FIXTURE_FILTER, (1.0, 0xFFFF, -3.0))
    prop(12, _lib.BODY_FIXED_ROTATION, 1.0)
    prop(9, _lib.BODY_BULLET, 1.0)
    prop(1, _lib.BODY_SLEEPING_ALLOWED, 0.0)
    prop(11, _lib.BODY_ANGULAR_DAMPING, 0.3)
    prop(5, _lib.BODY_MASS_DATA, (3.0, 0.2, -0.1, 2.5))
    step(20)
    prop(6, _lib.BODY_MASS_DATA, (3.0, 0.2, -0.1, 2.5))
    prop(6, _lib.BODY_RESET_MASS_DATA, 0.0)
    step(20)
    assert int(out["ends"][0]) == ends and ends > 0
    f32 = np.float32
    for ln in r.stdout.strip().splitlines():
        parts = ln.split()
        if parts[0] != "info":
            continue
        i = int(parts[1])
        got = np.array([float.fromhex(v) for v in parts[2:9]], dtype=np.float32)
        want, fl = o.body_info(i)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (i, got, want)
        flags = [int(x) for x in parts[9:14]]
        assert flags == [fl & 3, (fl >> 2) & 1, (fl >> 3) & 1, (fl >> 4) & 1, (fl >> 5) & 1], (i, flags, fl)
    # frame conversions of the bob (body 11) from its state, in the reference's operation order
    s = o.bodies()[11]
    px, py, cx, cy, vx, vy, w, sn, cs = s[0], s[1], s[3], s[4], s[5], s[6], s[7], s[8], s[9]
    lx, ly, gx, gy = f32(0.5), f32(0.25), f32(7.0), f32(3.0)
    wp = (f32(cs * lx - sn * ly) + px, f32(sn * lx + cs * ly) + py)
    wv = (f32(cs * lx - sn * ly), f32(sn * lx + cs * ly))
    qx, qy = f32(gx - px), f32(gy - py)
    lp = (f32(cs * qx + sn * qy), f32(-sn * qx + cs * qy))
    lv = (f32(cs * gx + sn * gy), f32(-sn * gx + cs * gy))
    vw = (vx + f32(-w * f32(gy - cy)), vy + f32(w * f32(gx - cx)))
    vl = (vx + f32(-w * f32(wp[1] - cy)), vy + f32(w * f32(wp[0] - cx)))
    want = np.array([*wp, *wv, *lp, *lv, *vw, *vl], dtype=np.float32)
    got = np.array([float.fromhex(v) for v in out["frames"]], dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (got, want)
    ob = o.bodies()
    assert len(bodies) == len(ob)
    for i, got in bodies.items():
        want = ob[i][[0, 1, 2, 5, 6, 7]]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i


JS_SRC = os.path.join(ROOT, "tests", "cpp", "joint_setters.cpp")


def _compile_js(tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "joint_setters")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), JS_SRC, "-o", exe,
           "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_joint_setters_compile(tmp_path):
    _compile_js(tmp_path)


def _js_scene():
    s = scenes.Scene(name="joint_setters")
    g = s.body(scenes.STATIC, 0.0, 0.0)
    s.fixture(g, scenes.EDGE, [-20.0, 0.0, 20.0, 0.0, 0, 0, 0, 0, 0, 0])
    p = s.body(scenes.DYNAMIC, 0.0, 5.0)
    s.fixture(p, scenes.BOX, [0.25, 1.0], 2, density=1.0)
    s.revolute(g, p, [0.0, 6.0], [0.0, 1.0])
    sl = s.body(scenes.DYNAMIC, 5.0, 2.0)
    s.fixture(sl, scenes.BOX, [0.5, 0.25], 2, density=1.0)
    s.prismatic(g, sl, [5.0, 2.0], [0.0, 0.0], [1.0, 0.0], lower=-1.0, upper=1.0, flags=1)
    ch = s.body(scenes.DYNAMIC, -8.0, 1.5)
    s.fixture(ch, scenes.BOX, [1.0, 0.25], 2, density=1.0)
    wh = s.body(scenes.DYNAMIC, -8.5, 0.6)
    s.fixture(wh, scenes.CIRCLE, [0.0, 0.0, 0.4], density=1.0)
    s.wheel(ch, wh, [-0.5, -0.9], [0.0, 0.0], [0.0, 1.0], max_motor_torque=20.0, motor_speed=0.0, frequency_hz=4.0,
            damping_ratio=0.7, flags=2)
    c1 = s.body(scenes.DYNAMIC, 10.0, 6.0)
    s.fixture(c1, scenes.CIRCLE, [0.0, 0.0, 0.3], density=1.0)
    c2 = s.body(scenes.DYNAMIC, 11.0, 6.0)
    s.fixture(c2, scenes.CIRCLE, [0.0, 0.0, 0.3], density=1.0)
    s.distance(c1, c2, [0.0, 0.0], [0.0, 0.0], 1.0)
    h = s.body(scenes.DYNAMIC, -3.0, 3.0)
    s.fixture(h, scenes.BOX, [0.3, 0.3], 2, density=1.0)
    s.motor(g, h, [-3.0, 3.0], 0.0, 100.0, 10.0, 0.3)
    return s


@pytest.mark.gpu
def test_cpp_joint_setters_match_oracle(gpu, tmp_path):
    """The typed joints of the C++ mirror (revolute, prismatic, wheel, distance, motor) and their
    setters against the CPU oracle with the same changes: every body bit for bit."""
    exe = _compile_js(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    rev = lines[0].split()
    assert rev[1:3] == ["1", "1"] and [float.fromhex(v) for v in rev[3:]] == [2.0, 100.0, -0.5, 0.5]
    o = oracle.OracleWorld(_js_scene(), "port", "project")
    for _ in range(30):
        o.step(1.0 / 60.0, 8, 3)
    for j, prop, v in [(0, 2, 1.0), (0, 0, 2.0), (0, 1, 100.0), (0, 4, (-0.5, 0.5)), (0, 3, 1.0),
                       (1, 2, 1.0), (1, 0, -1.5), (1, 1, 50.0), (1, 4, (-2.0, 0.5)),
                       (2, 0, -15.0), (2, 1, 60.0), (2, 6, 2.5), (2, 7, 0.4),
                       (3, 5, 1.6), (3, 6, 3.0), (3, 7, 0.2),
                       (4, 11, (-2.0, 4.0)), (4, 12, 0.5), (4, 9, 300.0), (4, 10, 200.0), (4, 13, 0.5)]:
        o.joint_set(j, prop, v)
    for _ in range(60):
        o.step(1.0 / 60.0, 8, 3)
    ob = o.bodies()
    reactions = 0
    for ln in lines[1:]:
        parts = ln.split()
        i = int(parts[1])
        got = np.array([float.fromhex(v) for v in parts[2:]], dtype=np.float32)
        if parts[0] == "reaction":
            assert np.array_equal(got.view(np.uint32), o.joint_reaction(i, 60.0).view(np.uint32)), ("joint", i)
            reactions += 1
            continue
        assert np.array_equal(got.view(np.uint32), ob[i][[0, 1, 2, 5, 6, 7]].view(np.uint32)), i
    assert reactions == 5


LISTS_SRC = os.path.join(ROOT, "tests", "cpp", "lists.cpp")


def test_cpp_lists_and_user_data(tmp_path):
    """b2Body::GetFixtureList / b2Fixture::GetNext and b2World::GetJointList / b2Joint::GetNext run
    newest first and skip destroyed entries, as the reference's lists; user data round-trips; the joint
    definitions' Initialize computes the reference's local anchors, axes, lengths and angles. No step
    is taken, so this runs without a GPU."""
    lib = _lib.library_path()
    exe = str(tmp_path / "lists")
    libdir = os.path.dirname(lib)
    # without contraction: the definitions' Initialize runs in the caller's code, compared bit for bit
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           LISTS_SRC, "-o", exe,
           "-L", libdir, "-lbox2d_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.strip().splitlines()}
    assert out["fixtures"] == ["2", "1", "0"]
    assert out["joints"] == ["2", "1", "0"]
    assert out["fixtures_after"] == ["2", "0"]
    assert out["joints_after"] == ["2", "0"]
    assert out["user"] == ["7", "8", "9"]
    assert out["ground_fixtures"] == ["3"]
    assert out["body_joints"] == ["2:0", "0:0"]  # newest first, the destroyed joint left out
    assert out["ground_contacts"] == ["0", "0"]  # no step yet: no contacts
    # the joint definitions' Initialize, restated in float32 from the printed transforms
    f32 = np.float32
    xfs = [[f32(float.fromhex(v)) for v in ln.split()[1:]] for ln in r.stdout.splitlines() if ln.startswith("xf ")]

    def local_point(t, p):
        dx, dy = f32(p[0] - t[0]), f32(p[1] - t[1])
        return [f32(t[3] * dx + t[2] * dy), f32(-t[2] * dx + t[3] * dy)]

    def local_vector(t, v):
        return [f32(t[3] * v[0] + t[2] * v[1]), f32(-t[2] * v[0] + t[3] * v[1])]

    a, c = xfs
    anchor, anchor2, axis = (f32(0.3), f32(1.1)), (f32(-1.7), f32(2.9)), (f32(0.6), f32(0.8))
    ref = f32(c[4] - a[4])
    dx, dy = f32(anchor2[0] - anchor[0]), f32(anchor2[1] - anchor[1])
    want = {
        "rev": local_point(a, anchor) + local_point(c, anchor) + [ref],
        "pri": local_point(a, anchor) + local_point(c, anchor) + local_vector(a, axis) + [ref],
        "whe": local_point(a, anchor) + local_point(c, anchor) + local_vector(a, axis),
        "dis": local_point(a, anchor) + local_point(c, anchor2) + [np.sqrt(f32(f32(dx * dx) + f32(dy * dy)), dtype=np.float32)],
        "mot": local_point(a, (c[0], c[1])) + [ref],
    }
    for key, vals in want.items():
        got = np.array([float.fromhex(v) for v in out[key]], dtype=np.float32)
        assert np.array_equal(got.view(np.uint32), np.array(vals, dtype=np.float32).view(np.uint32)), key
    assert out["weld_user"] == ["9"]
    # polygons after Set and SetAsBox(hx, hy, center, angle), as the library builds them
    polys = [ln.split()[1:] for ln in r.stdout.splitlines() if ln.startswith("poly ")]
    lib = _lib.load()
    for mode, inp, n, got in [(0, [0.0, 0.0, 1.5, 0.2, 0.7, 1.1, 0.6, 0.5, -0.4, 0.9], 5, polys[0]),
                              (2, [0.5, 0.25, 1.0, -2.0, 0.7], 0, polys[1])]:
        v = np.zeros(16, dtype=np.float32)
        v[:len(inp)] = inp
        o = np.zeros(34, dtype=np.float32)
        cnt = C.c_int()
        lib.gb_polygon_shape(mode, v, n, o, C.byref(cnt))
        assert int(got[0]) == cnt.value
        want = [o[0], o[1]] + [x for i in range(cnt.value) for x in (o[2 + 2 * i], o[3 + 2 * i], o[18 + 2 * i], o[19 + 2 * i])]
        vals = np.array([float.fromhex(x) for x in got[1:]], dtype=np.float32)
        assert np.array_equal(vals.view(np.uint32), np.array(want, dtype=np.float32).view(np.uint32))
