"""A user contact filter (b2World::SetContactFilter) on the device: the callback decides each ordered
fixture pair once; steps whose speculative default verdicts turn out wrong run again from their start,
so every step equals the reference running the same b2ContactFilter; a filter that agrees with the
default never re-runs a step and computes the default filter's bits."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib, scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, digest, golden

pytestmark = pytest.mark.gpu


def test_contact_filter_bit_exact_vs_reference(gpu):
    g = golden("filter_rule_project")
    sc = scenes.drop(200, scenes.SplitMix64(29))
    w = World(sc)
    ff = sc.arrays()["fix_filt"]

    def default(a, b):
        ca, ma, ga = int(ff[a][0]), int(ff[a][1]), int(ff[a][2])
        cb, mb, gb = int(ff[b][0]), int(ff[b][1]), int(ff[b][2])
        if ga == gb and ga != 0:
            return ga > 0
        return (ma & cb) != 0 and (ca & mb) != 0

    calls = []

    def should_collide(world, a, b):
        calls.append((a, b))
        return default(a, b) if a < 4 or b < 4 else (a + b) % 5 != 0

    w.set_contact_filter(should_collide)
    for s in range(1, int(g["steps"]) + 1):
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"
    replays, verdicts = w.filter_stats()
    assert replays > 0 and verdicts == len(calls) == len(set(calls))


def test_default_agreeing_filter_never_replays(gpu):
    sc = scenes.drop(150, scenes.SplitMix64(30))
    a, b = World(sc), World(sc)
    b.set_contact_filter(lambda w, fa, fb: True)  # every fixture has category 1, mask 0xFFFF, group 0
    for _ in range(90):
        a.step(DT, VI, PI)
        b.step(DT, VI, PI)
    a.sync(); b.sync()
    assert np.array_equal(a.bodies().view(np.uint32), b.bodies().view(np.uint32))
    assert b.filter_stats()[0] == 0


def test_cpp_contact_filter_matches_oracle(gpu, tmp_path):
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    lib = _lib.library_path()
    exe = str(tmp_path / "filter")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(root, "include"),
           os.path.join(root, "tests", "cpp", "filter.cpp"), "-o", exe, "-L", libdir, "-lbox2d_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    got = {int(ln.split()[1]): np.array([float.fromhex(v) for v in ln.split()[2:]], np.float32)
           for ln in lines if ln.startswith("body")}
    assert int(lines[-1].split()[1]) > 0
    sc = scenes.Scene(name="filter_cpp")
    gb = sc.body(scenes.STATIC, 0.0, 0.0)
    sc.fixture(gb, scenes.EDGE, [-20.0, 0.0, 20.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    pos = [(float(np.float32(-1.875 + r * 0.625 + j * 1.25)), 0.5 + r * 1.0) for r in range(3) for j in range(4 - r)]
    pos += [(-1.5 + 1.0 * k, 5.0 + 1.5 * k) for k in range(4)]
    for x, y in pos:
        b = sc.body(scenes.DYNAMIC, x, y)
        sc.fixture(b, scenes.BOX, [0.5, 0.5], 2, density=5.0, friction=0.6)
    o = oracle.OracleWorld(sc, "port", "project")
    o.set_filter_rule(5, 1)
    for _ in range(120):
        o.step(DT, VI, PI)
    ob = o.bodies()
    for i, v in got.items():
        assert np.array_equal(v.view(np.uint32), ob[i][[0, 1, 2, 5, 6, 7]].view(np.uint32)), i
