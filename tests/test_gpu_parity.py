"""GPU parity: the device step against the reference's golden vectors and the CPU oracle.

Bit-exact throughout: every step's full state (bodies, contact list order, manifolds, impulses,
flags) must equal, byte for byte, the reference Box2D 2.3.2 linked against the project trig. Against
the reference with glibc trig the same trajectories match at the start and stay within a stated
tolerance over the checkpoints (the project sin/cos differs from glibc's in ~1% of calls)."""
import numpy as np
import pytest

import oracle
from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World, collide, sincos
from tests._util import DT, PI, VI, digest, first_divergence, golden, trajectory_cases

CASES = trajectory_cases()
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,make,steps", CASES, ids=[c[0] for c in CASES])
def test_gpu_trajectory_bit_exact_vs_reference(gpu, name, make, steps):
    g = golden(f"{name}_project")
    w = World(make())
    bad = first_divergence(w, steps, g["digests"])
    assert bad is None, f"{name}: GPU state first differs from the reference at step {bad}"
    w.sync()


def test_gpu_batched_worlds_bit_exact(gpu):
    """All 24 sample worlds of the batched workload in ONE batch (one CTA per world)."""
    worlds = scenes.config3(24, seed=9)
    gold = [golden(f"batch{i}_project") for i in range(24)]
    w = World(worlds)
    for s in range(1, 201):
        w.step(DT, VI, PI)
        if s % 20 == 0 or s == 1:
            for i in range(24):
                b = w.bodies(i)
                ci, cf = w.contacts(i)
                assert np.array_equal(digest(b, ci, cf), gold[i]["digests"][s - 1]), (i, s)
    w.sync()


def test_gpu_pyramid_close_to_glibc_reference(gpu):
    """Against the reference as shipped (glibc sin/cos): position error bound at checkpoints."""
    g = golden("pyramid20_libm")
    w = World(scenes.config1())
    for s in range(1, 601):
        w.step()
        if s in (1, 10, 60, 120, 300, 600):
            b = w.bodies()[1:]
            ref = g[f"bodies_{s}"][1:]
            err = np.abs(b[:, 0:2] - ref[:, 0:2]).max()
            assert err < 2e-3, (s, err)


def test_gpu_collide_matches_reference(gpu):
    g = golden("collide")
    oi, of = collide(g["type_a"], g["shape_a"], g["n_a"], g["xf_a"], g["type_b"], g["shape_b"], g["n_b"], g["xf_b"])
    assert np.array_equal(oi, g["out_ints"])
    assert np.array_equal(of.view(np.uint32), g["out_floats"].view(np.uint32))


def test_gpu_sincos_equals_oracle_trig(gpu):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-10, 10, 200000), rng.uniform(-1e-3, 1e-3, 50000),
                        rng.uniform(-1e6, 1e6, 50000), np.array([0.0, -0.0, 1e-30, -1e-30, 3e8, -3e8])]).astype(np.float32)
    s, c = sincos(x)
    lib = oracle.load("port", "project")
    idx = np.arange(0, len(x), 13)
    for i in idx:
        rs, rc = oracle.sincosf("port", "project", float(x[i]))
        assert np.float32(rs).view(np.uint32) == s[i].view(np.uint32) and np.float32(rc).view(np.uint32) == c[i].view(np.uint32), x[i]


@pytest.mark.parametrize("seed", [31, 32])
def test_gpu_matches_oracle_on_fresh_drops(gpu, seed):
    """Seeds with no golden file: the CPU oracle (project trig) is the checker."""
    sc = scenes.drop(700, scenes.SplitMix64(seed), allow_sleep=(seed % 2 == 0))
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 151):
        w.step(); o.step()
        if s % 10 == 0:
            gb, ob = w.bodies(), o.bodies()
            gi, gf = w.contacts()
            oi, of = o.contacts()
            assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), s
            assert np.array_equal(gi, oi) and np.array_equal(gf.view(np.uint32), of.view(np.uint32)), s


def test_gpu_large_world_sweep_pairs_match_oracle(gpu):
    """One world of 10,000 circles and polygons (the 200 m container mix): the broadphase takes the
    sort-and-sweep path (more than 2^20 candidate tests), which must find the reference's pair set;
    every body and contact matches the CPU oracle bit for bit at checkpoints."""
    sc = scenes.config2(10000, seed=1, allow_sleep=True)
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 41):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        if s in (1, 2, 5, 10, 20, 40):
            gb, ob = w.bodies(0), o.bodies()
            assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ at step {s}"
            gi, gf = w.contacts(0)
            oi, of = o.contacts()
            assert np.array_equal(gi, oi), f"contacts differ at step {s}"
            assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), f"manifolds differ at step {s}"
    w.sync()


def test_gpu_toi_event_loop_matches_oracle(gpu):
    """A drop whose fast bodies hit the container: many steps take several time-of-impact events, so
    the event loop's later events (only the contacts an event touched are classified again) run
    often; every body and contact matches the CPU oracle bit for bit after every step."""
    sc = scenes.drop(400, scenes.SplitMix64(11), allow_sleep=False)
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    events, multi = 0, 0
    for s in range(1, 121):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        e = w.stats(0)[1]
        events += e
        multi += e >= 2
        gb, ob = w.bodies(0), o.bodies()
        assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ at step {s}"
        gi, gf = w.contacts(0)
        oi, of = o.contacts()
        assert np.array_equal(gi, oi), f"contacts differ at step {s}"
        assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), f"manifolds differ at step {s}"
    w.sync()
    assert events >= 20 and multi >= 5, (events, multi)


def test_gpu_grid_pair_finding_matches_oracle(gpu):
    """3,000 bodies dropped into the edge container with sleep off: every step's pair finding has more
    than 2^20 candidate tests and bins the proxies into a grid; the pair set, and so every body and
    contact, must match the CPU oracle bit for bit through the fall and the pile-up."""
    sc = scenes.config2(3000, seed=4, allow_sleep=False)
    w = World(sc)
    o = oracle.OracleWorld(sc, "port", "project")
    for s in range(1, 151):
        w.step(DT, VI, PI)
        o.step(DT, VI, PI)
        if s % 15 == 0:
            gb, ob = w.bodies(0), o.bodies()
            assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32)), f"bodies differ at step {s}"
            gi, gf = w.contacts(0)
            oi, of = o.contacts()
            assert np.array_equal(gi, oi), f"contacts differ at step {s}"
            assert np.array_equal(gf.view(np.uint32), of.view(np.uint32)), f"manifolds differ at step {s}"
    w.sync()
