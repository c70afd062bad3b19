"""gb_collide_noalloc (narrowphase staged in the library's fixed device buffer) against gb_collide.

Collected last (file name), so the in-process cases run after every other test has used the
library; one case runs in a fresh process so the buffer's first use there is covered too. Each case
makes two calls in a row to show the shared buffer is reused cleanly.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

from box2dpp_gb300 import _lib
from box2dpp_gb300.world import collide, collide_noalloc
from tests._util import golden

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
pytestmark = pytest.mark.gpu

KEYS = ("type_a", "shape_a", "n_a", "xf_a", "type_b", "shape_b", "n_b", "xf_b")


def _pairs(n=None):
    g = golden("collide")
    args = [g[k] for k in KEYS]
    if n is not None:
        reps = -(-n // len(args[0]))
        args = [np.concatenate([a] * reps)[:n] for a in args]
    return args


def _same(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


def test_noalloc_matches_collide_twice_after_other_tests(gpu):
    args = _pairs()
    ref = collide(*args)
    first = collide_noalloc(*args)
    second = collide_noalloc(*args)
    assert _same(first, ref)
    assert _same(second, ref)
    g = golden("collide")
    assert np.array_equal(first[0], g["out_ints"])


def test_noalloc_full_buffer_twice(gpu):
    args = _pairs(_lib.COLLIDE_NOALLOC_MAX_PAIRS)
    ref = collide(*args)
    assert _same(collide_noalloc(*args), ref)
    # a smaller call after a full one: stale buffer contents must not leak into the result
    small = [a[:1000][::-1].copy() for a in args]
    assert _same(collide_noalloc(*small), collide(*small))


FRESH = r"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
from box2dpp_gb300.world import collide, collide_noalloc
from tests._util import golden
g = golden("collide")
args = [g[k] for k in {keys!r}]
first = collide_noalloc(*args)      # the first library call of this process
second = collide_noalloc(*args)
ref = collide(*args)
for out in (first, second):
    assert np.array_equal(out[0], ref[0])
    assert np.array_equal(out[1].view(np.uint32), ref[1].view(np.uint32))
assert np.array_equal(first[0], g["out_ints"])
print("noalloc-fresh-ok")
"""


def test_noalloc_in_fresh_process(gpu):
    code = FRESH.format(root=ROOT, keys=KEYS)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "noalloc-fresh-ok" in r.stdout


def test_noalloc_rejects_oversized_and_invalid(gpu):
    args = _pairs(_lib.COLLIDE_NOALLOC_MAX_PAIRS + 1)
    with pytest.raises(_lib.GbError) as e:
        collide_noalloc(*args)
    assert e.value.status == _lib.GB_ERR_CAPACITY
    bad = _pairs(8)
    bad[0] = bad[0].copy()
    bad[4] = bad[4].copy()
    bad[0][3], bad[4][3] = 1, 1  # edge against edge: no collider
    with pytest.raises(_lib.GbError) as e:
        collide_noalloc(*bad)
    assert e.value.status == _lib.GB_ERR_INVALID
