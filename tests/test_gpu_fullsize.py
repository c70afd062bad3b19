"""Parity at the workloads' stated sizes: the 10,000-body drop through its pile-up, the
65,536-body stress world with 512 revolute chains, and the benchmark's own 4,096-world batch with
the launch plan its autotuner picks, stepped by CUDA-graph replay. The reference-order solver is
compared bit for bit with the CPU oracle (project trig) at checkpoints; the oracle steps in a host
thread while the device steps, so the two overlap. The graph-coloured arm of the benchmark is held
to the benchmark's own accuracy rule and to determinism."""
from __future__ import annotations

import os
import threading

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes, shard
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu

# the benchmark's steps before its timed window: the launch-plan autotuner's trials
PRE_STEPS = 24


def _same_world(w, i, o, where):
    gb, ob = w.bodies(i), o.bodies()
    assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ {where}"
    gi, gf = w.contacts(i)
    oi, of = o.contacts()
    assert np.array_equal(gi, oi), f"contact list differs {where}"
    assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), f"manifolds differ {where}"


def _advance(worlds, steps, threads=1):
    """The oracle worlds stepped `steps` times in a host thread (returned, already started)."""
    th = threading.Thread(target=oracle.step_many, args=(worlds, steps, threads, DT, VI, PI))
    th.start()
    return th


def _checkpointed(w, o, checkpoints):
    done = 0
    for cp in checkpoints:
        th = _advance([o], cp - done)
        for _ in range(cp - done):
            w.step(DT, VI, PI)
        w.sync()
        th.join()
        done = cp
        _same_world(w, 0, o, f"at step {cp}")


def test_config2_settled_pile_matches_oracle(gpu):
    """10,000 circles and polygons dropped into the 200 m edge box, sleep on (the reference default),
    through 600 steps: the fall and the pile-up (at step 600 the pile still moves, median speed about
    0.2 m/s)."""
    sc = scenes.config2(10000, seed=1, allow_sleep=True)
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    _checkpointed(w, o, [100, 300, 600])
    # the bodies have landed and piled up: several contacts per body
    ints, _ = w.contacts(0)
    assert len(ints) > 2 * 10000, len(ints)


def test_config5_full_size_matches_oracle(gpu):
    """65,536 bodies (60% boxes, 40% circles) with 512 chains of 16 revolute-jointed links in a 300 m
    container of kinematic edges spinning at 0.05 rad/s, sleep off, 120 steps."""
    sc = scenes.config5(allow_sleep=False)
    assert sc.dynamic_count >= 65536 and len(sc.joints) >= 512 * 15
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    _checkpointed(w, o, [1, 60, 120])


def _bench_batch(solver: str, vi: int, plan=None):
    ws = shard.shard_workload(4096, 1, 0, allow_sleep=False)
    w = World(ws)
    w.set_solver(solver, measure_residual=True)
    w.upload()
    if plan is None:
        w.autotune(2)
    else:
        w.set_launch_plan(plan)
    for _ in range(PRE_STEPS):
        w.step(DT, vi, PI)
    return ws, w


def test_bench_batch_plain_graph_matches_oracle(gpu):
    """The benchmark's batch (4,096 worlds, 568,923 bodies) with the reference-order solver: the
    autotuner's plan, then 30 graph-replayed steps; every world against the oracle on all host cores."""
    ws, w = _bench_batch("plain", VI)
    classes, ms = w.launch_plan()
    assert len(ms) > 0, "the autotuner did not finish within the benchmark's tuning steps"
    os_ = [oracle.OracleWorld(s, "port", "project") for s in ws]
    th = _advance(os_, PRE_STEPS + 30, os.cpu_count() or 1)
    for _ in range(30):
        w.graph_step(DT, VI, PI)
    w.sync()
    th.join()
    for i in range(len(ws)):
        _same_world(w, i, os_[i], f"in world {i} after {PRE_STEPS + 30} steps")


def test_bench_batch_coloured_accuracy_and_determinism(gpu):
    """The benchmark's headline arm: the graph-coloured solver at 10 velocity iterations on the same
    batch. Its median velocity residual must be no larger than the reference-order solver's at 8
    (the benchmark's matched-accuracy rule), and the tuned plan replayed from a CUDA graph must give
    the same bits as another plan stepped without a graph."""
    ws, a = _bench_batch("coloured", 10)
    plan, _ = a.launch_plan()
    _, b = _bench_batch("coloured", 10, plan=[[0, 4096, 64, 640, 1024]])
    _, p = _bench_batch("plain", VI, plan=plan)
    for _ in range(30):
        a.graph_step(DT, 10, PI)
        b.step(DT, 10, PI)
        p.graph_step(DT, VI, PI)
    a.sync(); b.sync(); p.sync()
    ra, rp = a.solver_stats()[2], p.solver_stats()[2]
    assert np.all(np.isfinite(ra))
    assert np.median(ra) <= np.median(rp), (np.median(ra), np.median(rp))
    for i in range(0, len(ws), 7):
        assert np.array_equal(a.bodies(i).view(np.uint32), b.bodies(i).view(np.uint32)), i
        ai, af = a.contacts(i)
        bi, bf = b.contacts(i)
        assert np.array_equal(ai, bi) and np.array_equal(af.view(np.uint32), bf.view(np.uint32)), i
    # no world blows up: the deepest penetration the position solver saw stays at body scale
    assert float(a.max_penetration().max()) < 2.0
