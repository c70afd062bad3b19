"""Shared helpers of the test-suite: golden fixture loading and state digests."""
from __future__ import annotations

import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DT, VI, PI = 1.0 / 60.0, 8, 3


def digest(bodies, ints, flts) -> np.ndarray:
    """SHA-256 of one step's full state in the dump layout (tests/golden/make_golden.py)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(bodies, dtype=np.float32).tobytes())
    h.update(np.ascontiguousarray(ints, dtype=np.int32).tobytes())
    h.update(np.ascontiguousarray(flts, dtype=np.float32).tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8)


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def trajectory_cases():
    """(name, scene factory, steps) of every golden trajectory, from the generator script."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return [(n, f, s) for (n, f, s, _c) in mod.cases()]


def first_divergence(world, steps: int, golden_digests: np.ndarray):
    """Step index (1-based) where `world`'s state digest first differs from the golden one, or None."""
    for s in range(1, steps + 1):
        world.step(DT, VI, PI)
        b = world.bodies()
        ci, cf = world.contacts()
        if not np.array_equal(digest(b, ci, cf), golden_digests[s - 1]):
            return s
    return None
