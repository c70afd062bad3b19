"""A step split at its collide phase for a PreSolve listener that changes contacts: the split itself
computes the same bits as a whole step, and with the listener's changes applied between the halves
(gb_contact_edits) the device follows the reference running the same listener, step by step; the C++
mirror does the same through its b2ContactListener."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, digest, golden, presolve_case, presolve_edits

pytestmark = pytest.mark.gpu
ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_split_step_without_changes_equals_step(gpu):
    sc = scenes.drop(300, scenes.SplitMix64(8))
    a, b = World(sc), World(sc)
    b.set_events(True)
    for _ in range(120):
        a.step(DT, VI, PI)
        b.step_begin(DT, VI, PI)
        b.step_end()
    a.sync(); b.sync()
    assert np.array_equal(a.bodies().view(np.uint32), b.bodies().view(np.uint32))
    ai, af = a.contacts()
    bi, bf = b.contacts()
    assert np.array_equal(ai, bi) and np.array_equal(af.view(np.uint32), bf.view(np.uint32))


def test_presolve_changes_bit_exact_vs_reference(gpu):
    g = golden("presolve_rule_project")
    sc, bits = presolve_case()
    w = World(sc)
    w.set_events(True)
    changed = 0
    for s in range(1, int(g["steps"]) + 1):
        w.step_begin(DT, VI, PI)
        edits = presolve_edits(w, bits)
        changed += len(edits)
        w.contact_edits(edits)
        w.step_end()
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    assert changed > 1000


def test_split_step_locks_the_world(gpu):
    w = World(scenes.pyramid(4))
    w.step_begin(DT, VI, PI)
    with pytest.raises(_lib.GbError):
        w.step(DT, VI, PI)
    with pytest.raises(_lib.GbError):
        w.destroy_body(1)
    w.step_end()
    with pytest.raises(_lib.GbError):
        w.step_end()
    w.step(DT, VI, PI)
    w.sync()


def test_cpp_presolve_listener_matches_oracle(gpu, tmp_path):
    lib = _lib.library_path()
    exe = str(tmp_path / "presolve")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "presolve.cpp"), "-o", exe, "-L", libdir, "-lbox2d_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    got = {int(ln.split()[1]): np.array([float.fromhex(v) for v in ln.split()[2:]], np.float32)
           for ln in lines if ln.startswith("body")}
    assert int(lines[-1].split()[1]) > 0
    sc = scenes.Scene(name="presolve_cpp")
    gb = sc.body(scenes.STATIC, 0.0, 0.0)
    sc.fixture(gb, scenes.EDGE, [-20.0, 0.0, 20.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    pos = [(float(np.float32(-1.875 + r * 0.625 + j * 1.25)), 0.5 + r * 1.0) for r in range(3) for j in range(4 - r)]
    pos += [(-1.5 + 1.0 * k, 5.0 + 1.5 * k) for k in range(4)]
    for x, y in pos:
        b = sc.body(scenes.DYNAMIC, x, y)
        sc.fixture(b, scenes.BOX, [0.5, 0.5], 2, density=5.0, friction=0.6)
    bits = np.array([0] + [(f % 3 == 0) * 1 | (f % 4 == 0) * 2 | (f % 5 == 0) * 4 for f in range(1, 14)], np.int32)
    o = oracle.OracleWorld(sc, "port", "project")
    o.set_presolve_rule(bits)
    for _ in range(120):
        o.step(DT, VI, PI)
    ob = o.bodies()
    for i, v in got.items():
        assert np.array_equal(v.view(np.uint32), ob[i][[0, 1, 2, 5, 6, 7]].view(np.uint32)), i
