"""The graph-coloured island solver against the plain (reference-order) solver on the GPU.

The coloured solver is not bit-exact with the reference (its Gauss-Seidel order differs), so it is
checked the way the solver variants are compared: the velocity residual it reaches, the physical
state it settles into, run-to-run determinism, and the iterations a residual tolerance saves.
"""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI

pytestmark = pytest.mark.gpu


def _run(scene_list, solver, steps, tolerance=0.0, vi=VI):
    w = World(scene_list)
    w.set_solver(solver, tolerance=tolerance, measure_residual=True)
    res, its, cols = [], [], []
    for _ in range(steps):
        w.step(DT, vi, PI)
        col, it, r = w.solver_stats()
        res.append(r.copy())
        its.append(it.copy())
        cols.append(col.copy())
    w.sync()
    return w, np.array(res), np.array(its), np.array(cols)


def test_coloured_pyramid_stands_like_plain(gpu):
    sc = scenes.pyramid(20)
    wp, rp, _, _ = _run(sc, "plain", 300)
    wc, rc, _, col = _run(sc, "coloured", 300)
    bp, bc = wp.bodies(0), wc.bodies(0)
    assert np.all(np.isfinite(bc))
    # same resting pile: every box within 5 cm of the plain solver's position after 5 s (the two
    # Gauss-Seidel orders drift apart by a few millimetres per row of a 20-row stack)
    assert np.max(np.abs(bp[:, 0:2] - bc[:, 0:2])) < 0.05
    assert np.max(np.abs(bc[:, 5:8])) < 0.05  # at rest
    assert 2 <= col[:, 0].max() < 63  # colours while awake (the pile may fall asleep)
    # matched accuracy: the coloured solver's residual over the settled steps is no worse than 2x plain's
    assert np.median(rc[100:]) <= 2.0 * np.median(rp[100:]) + 1e-5


def test_coloured_batch_deterministic_and_finite(gpu):
    ws = scenes.config3(64, seed=5, allow_sleep=False)
    a, ra, _, _ = _run(ws, "coloured", 60)
    b, rb, _, _ = _run(ws, "coloured", 60)
    for i in range(len(ws)):
        A, B = a.bodies(i), b.bodies(i)
        assert np.all(np.isfinite(A))
        assert np.array_equal(A.view(np.uint32), B.view(np.uint32)), i
    assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))


def test_tolerance_ends_velocity_iterations_early(gpu):
    ws = scenes.config3(32, seed=7, allow_sleep=False)
    for solver in ("plain", "coloured"):
        _, r_full, it_full, _ = _run(ws, solver, 120, 0.0, 30)
        _, r_tol, it_tol, _ = _run(ws, solver, 120, 1e-2, 30)
        assert np.all(it_full[-1] == 30)
        assert it_tol[60:].mean() < 30
        assert np.all(it_tol <= 30)


def test_plain_solver_unchanged_by_residual_measurement(gpu):
    sc = scenes.pyramid(8)
    a = World(sc)
    b = World(sc)
    b.set_solver("plain", measure_residual=True)
    for _ in range(60):
        a.step(DT, VI, PI)
        b.step(DT, VI, PI)
    assert np.array_equal(a.bodies(0).view(np.uint32), b.bodies(0).view(np.uint32))
