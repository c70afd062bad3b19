"""b2PolygonShape::Set and SetAsBox as the library stores a polygon (gb_polygon_shape: hull of welded
points, vertices, normals, centroid), against the compiled reference's own b2PolygonShape (project trig
for the rotated box), for seeded point clouds, degenerate inputs and boxes. No GPU is needed."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

import oracle
from box2dpp_gb300 import _lib


def _ours(mode, inp, n):
    lib = _lib.load()
    out = np.zeros(34, dtype=np.float32)
    cnt = C.c_int()
    v = np.zeros(16, dtype=np.float32)
    v[:len(inp)] = inp
    _lib.check(lib.gb_polygon_shape(mode, v, n, out, C.byref(cnt)), "gb_polygon_shape")
    return out, cnt.value


def _reference(mode, inp, n):
    path = os.path.join(os.path.dirname(oracle.__file__), "_ref", "libref_proj.so")
    lib = C.CDLL(path)
    fn = lib.rw_polygon_shape
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, np.ctypeslib.ndpointer(np.float32), C.c_int, np.ctypeslib.ndpointer(np.float32)]
    v = np.zeros(16, dtype=np.float32)
    v[:len(inp)] = inp
    out = np.zeros(34, dtype=np.float32)
    return out, fn(mode, v, n, out)


def _cases():
    rng = np.random.default_rng(5)
    cases = []
    for k in range(60):
        n = int(rng.integers(3, 9))
        pts = rng.uniform(-2.0, 2.0, size=2 * n).astype(np.float32)
        if k % 10 == 0:
            pts[2:4] = pts[0:2] + np.float32(1e-4)  # two points welded
        cases.append((0, pts, n))
    cases.append((0, np.array([0, 0, 1, 0, 2, 0, 3, 0], np.float32), 4))  # collinear: no hull
    cases += [(1, np.array([0.5, 1.25], np.float32), 0), (2, np.array([0.5, 0.25, 1.0, -2.0, 0.7], np.float32), 0),
              (2, np.array([3.0, 0.1, -5.5, 0.25, -2.2], np.float32), 0)]
    return cases


@pytest.mark.parametrize("case", range(len(_cases())))
def test_polygon_shape_matches_reference(case):
    if not oracle.reference_available():
        pytest.skip("reference tree not present")
    oracle.build_reference()
    mode, inp, n = _cases()[case]
    a, na = _ours(mode, inp, n)
    b, nb = _reference(mode, inp, n)
    assert na == nb
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (a, b)
