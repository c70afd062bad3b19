"""Launch plans and the online autotuner: every plan must compute the same bits."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _state(w):
    out = []
    for i in range(w.n_worlds):
        ints, flts = w.contacts(i)
        out.append((w.bodies(i).view(np.uint32).copy(), ints.copy(), flts.view(np.uint32).copy()))
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for p, q in zip(a, b) for x, y in zip(p, q))


@pytest.mark.parametrize("solver", ["plain", "coloured"])
def test_plans_compute_identical_bits(gpu, solver):
    ws = scenes.config3(48, seed=11, allow_sleep=True)
    runs = []
    for plan in (None, "split", "tiny"):
        w = World(ws)
        w.set_solver(solver)
        w.upload()
        if plan == "split":
            w.set_launch_plan([[0, 10, 128, 640, 1024], [10, 20, 64, 256, 512], [30, 18, 32, 128, 256]])
        elif plan == "tiny":
            # shared memory far too small for most worlds: every staging falls back to global memory
            w.set_launch_plan([[0, 48, 32, 16, 16]])
        for _ in range(80):
            w.step(DT, VI, PI)
        w.sync()
        runs.append(_state(w))
    assert _same(runs[0], runs[1])
    assert _same(runs[0], runs[2])


def test_autotune_chooses_a_candidate_without_changing_results(gpu):
    ws = scenes.config3(96, seed=12, allow_sleep=False)
    a, b = World(ws), World(ws)
    a.upload()
    b.upload()
    b.autotune(1)
    steps = 0
    while True:
        a.step(DT, VI, PI)
        b.step(DT, VI, PI)
        steps += 1
        classes, ms = b.launch_plan()
        if len(ms) > 0 or steps > 64:
            break
    assert len(ms) >= 2 and np.all(ms > 0)
    assert classes[:, 1].sum() == 96 and classes[0, 0] == 0
    for _ in range(20):
        a.step(DT, VI, PI)
        b.step(DT, VI, PI)
    assert _same(_state(a), _state(b))


def test_bad_plans_are_rejected(gpu):
    from box2dpp_gb300 import _lib

    w = World(scenes.config3(8, seed=1))
    w.upload()
    for bad in ([[0, 7, 64, 64, 64]], [[1, 8, 64, 64, 64]], [[0, 8, 48, 64, 64]], [[0, 8, 64, 4096, 4096]]):
        with pytest.raises(_lib.GbError):
            w.set_launch_plan(bad)


@pytest.mark.parametrize("solver", ["plain", "coloured"])
def test_graph_step_matches_step(gpu, solver):
    ws = scenes.config3(40, seed=13, allow_sleep=True)
    a, b = World(ws), World(ws)
    for w in (a, b):
        w.set_solver(solver)
        w.upload()
    # a three-class plan: the captured graph holds the forked side-stream launches too
    b.set_launch_plan([[0, 8, 64, 640, 1024], [8, 16, 64, 256, 512], [24, 16, 32, 128, 256]])
    for _ in range(50):
        a.step(DT, VI, PI)
        b.graph_step(DT, VI, PI)
    b.sync()
    assert _same(_state(a), _state(b))


def test_pipelined_transfers_match_synchronous_ones(gpu):
    """gb_set_forces_async / gb_get_transforms_async in a graph-replayed loop give the bits of
    gb_set_forces / gb_get_transforms with a step between them (per-step forces differ, so a late or
    early upload would show)."""
    import torch

    ws = scenes.config3(24, seed=17, allow_sleep=False)
    a, b = World(ws), World(ws)
    for w in (a, b):
        w.set_solver("coloured")
        w.upload()
    n = a.total_bodies
    rng = np.random.default_rng(5)
    forces = [rng.normal(0.0, 20.0, (n, 4)).astype(np.float32) for _ in range(12)]
    host_f = [torch.from_numpy(f).pin_memory() for f in forces]
    host_x = [torch.zeros((n, 4), dtype=torch.float32).pin_memory() for _ in forces]
    sync_x = []
    for k in range(len(forces)):
        a.set_forces_ptr(host_f[k].data_ptr())
        a.graph_step(DT, VI, PI)
        sync_x.append(a.get_transforms())
    for k in range(len(forces)):
        b.set_forces_async_ptr(host_f[k].data_ptr())
        b.graph_step(DT, VI, PI)
        b.get_transforms_async_ptr(host_x[k].data_ptr())
    b.sync()
    for k in range(len(forces)):
        assert np.array_equal(sync_x[k].view(np.uint32), host_x[k].numpy().view(np.uint32)), k
    assert not np.array_equal(sync_x[0], sync_x[-1])


@pytest.mark.parametrize("solver", ["plain", "coloured"])
def test_wide_ctas_compute_identical_bits(gpu, solver):
    """One world on CTAs of 128, 256 and 512 threads (the widths a single world's plans use)."""
    sc = scenes.config2(1500, seed=3, allow_sleep=False)
    runs = []
    for threads in (128, 256, 512):
        w = World([sc])
        w.set_solver(solver)
        w.upload()
        w.set_launch_plan([[0, 1, threads, 640, 1024]])
        for _ in range(60):
            w.step(DT, VI, PI)
        w.sync()
        runs.append(_state(w))
        w.close()
    assert _same(runs[0], runs[1]) and _same(runs[0], runs[2])
