"""Generate the golden vectors under tests/golden/ from the UNMODIFIED reference (box2dref compiled by
oracle/Makefile from the reference tree). Run where the reference tree exists:

    python tests/golden/make_golden.py [--queries]

Two builds of the reference are used: ``libm`` (glibc sinf/cosf, the reference as shipped) and
``project`` (the same objects with sinf/cosf/sincosf resolved to the project trig). Fixtures:

* ``<case>_<trig>.npz``: for a scene stepped N times, the SHA-256 of every step's full state
  (bodies 12 x float32 + contacts 8 x int32 + 12 x float32 in world-list order, as dumped by the
  C-ABIs) and the full body/contact arrays at a few checkpoint steps (none for the 10,000-body
  drop, whose arrays would be megabytes).

  python tests/golden/make_golden.py --case <name>   writes one trajectory case only.
* ``destroy_mix_<trig>.npz``: a scene changed between steps (bodies, joints and fixtures destroyed,
  bodies created) with the per-step digests, the destruction listener's calls and the final proxy
  ids (freed tree nodes are reused).
* ``presolve_rule_<trig>.npz``: a drop with a PreSolve listener that disables, de-frictions or
  bounces contacts by a per-fixture rule (tests/_util.py presolve_case), per-step digests.
* ``filter_rule_<trig>.npz``: a drop with a user b2ContactFilter (walls default; other pairs collide
  unless (fixtureA + fixtureB) % 5 == 0), per-step digests.
* ``collide.npz``: seeded shape pairs of every supported type pair with the reference manifolds.
* ``toi.npz``: seeded sweeps with the reference b2TimeOfImpact result.
* ``trig.npz``: glibc sinf/cosf on seeded angles (how far the project trig is from libm).
* ``fixture_queries.npz``: b2Fixture::TestPoint, RayCast and GetAABB of every fixture of a stepped
  scene for seeded points and rays (``--fixture-queries`` writes only this file).
* ``tree_stats.npz``: b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality after every step of
  trajectory and scripted cases (project trig; ``--tree`` writes only this file).
* ``query_<scene>.npz``: b2World::QueryAABB and closest-hit b2World::RayCast results on a stepped
  scene (project trig) for seeded boxes and segments (``--queries`` writes only these).
"""
from __future__ import annotations

import hashlib
import math
import zlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

import oracle  # noqa: E402
from box2dpp_gb300 import scenes  # noqa: E402

DT, VI, PI = 1.0 / 60.0, 8, 3


def state_digest(bodies: np.ndarray, ints: np.ndarray, flts: np.ndarray) -> bytes:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(bodies, dtype=np.float32).tobytes())
    h.update(np.ascontiguousarray(ints, dtype=np.int32).tobytes())
    h.update(np.ascontiguousarray(flts, dtype=np.float32).tobytes())
    return h.digest()


_BATCH = []


def batch_world(i: int):
    """World i of the 24-world batched sample (seed 9)."""
    if not _BATCH:
        _BATCH.extend(scenes.config3(24, seed=9))
    return _BATCH[i]


def cases():
    """Named trajectory cases: (name, scene factory, steps, checkpoints)."""
    return [
        ("pyramid20", lambda: scenes.config1(), 600, [1, 10, 60, 120, 300, 600]),
        ("drop300", lambda: scenes.drop(300, scenes.SplitMix64(7)), 300, [1, 30, 100, 300]),
        ("drop1000_nosleep", lambda: scenes.drop(1000, scenes.SplitMix64(21), allow_sleep=False), 120, [1, 60, 120]),
        ("stacks120", lambda: scenes.stacks(120, scenes.SplitMix64(5)), 300, [1, 150, 300]),
        ("chains6x16", lambda: chains_with_load(), 300, [1, 100, 300]),
        ("joint_mix", lambda: scenes.joint_mix(scenes.SplitMix64(3)), 300, [1, 60, 150, 300]),
        ("prismatic_mix", lambda: scenes.prismatic_mix(scenes.SplitMix64(5)), 300, [1, 60, 150, 300]),
        ("joint_zoo", lambda: scenes.joint_zoo(scenes.SplitMix64(6)), 300, [1, 60, 150, 300]),
        ("pulley_mouse", lambda: scenes.pulley_mouse(scenes.SplitMix64(4)), 300, [1, 60, 150, 300]),
        ("gears", lambda: scenes.gears(scenes.SplitMix64(8)), 300, [1, 60, 150, 300]),
        ("chain_terrain", lambda: scenes.chain_terrain(scenes.SplitMix64(12)), 300, [1, 60, 150, 300]),
        ("sensors", lambda: scenes.sensors(scenes.SplitMix64(13)), 300, [1, 100, 300]),
        # the 10,000-body drop at full size: per-step digests only (no checkpoint arrays, which would
        # be megabytes)
        ("config2_10k", lambda: scenes.config2(10000, seed=1, allow_sleep=True), 200, []),
    ] + [(f"batch{i}", (lambda i=i: batch_world(i)), 200, [200]) for i in range(24)]


def scripted_cases():
    """Trajectory cases with b2World changes between steps: (name, scene factory, steps, ops by step).
    The ops (tests/_util.py destroy_script) destroy bodies, joints and fixtures and create bodies."""
    sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
    from tests._util import (body_props_script, destroy_script, fixture_props_script, joint_scripts, settings_script,
                             shift_script)

    return [("destroy_mix", lambda: scenes.destroy_mix(scenes.SplitMix64(5)), 200, destroy_script()),
            ("settings_mix", lambda: scenes.destroy_mix(scenes.SplitMix64(7)), 340, settings_script()),
            ("body_props", lambda: scenes.destroy_mix(scenes.SplitMix64(11)), 320, body_props_script()),
            ("fixture_props", lambda: scenes.destroy_mix(scenes.SplitMix64(13)), 300, fixture_props_script()),
            ("shift_origin", lambda: scenes.pulley_mouse(scenes.SplitMix64(4)), 260, shift_script())] + \
        [(name, make, steps, script) for name, (make, steps, script) in joint_scripts().items()]


def run_scripted(scene, steps, script, trig):
    """Per-step state digests, the destruction listener's calls as (step, kind, index) rows and the
    final proxy ids and fat AABBs of the reference on a scripted case."""
    from tests._util import apply_ops

    w = oracle.OracleWorld(scene, "reference", trig)
    digests = np.zeros((steps, 32), dtype=np.uint8)
    calls = []
    for s in range(1, steps + 1):
        if s in script:
            calls += [(s, k, i) for (k, i) in apply_ops(w, script[s])]
        w.step(DT, VI, PI)
        b = w.bodies()
        ci, cf = w.contacts()
        digests[s - 1] = np.frombuffer(state_digest(b, ci, cf), dtype=np.uint8)
    ids, fat = w.proxies()
    return digests, np.array(calls, np.int32).reshape(-1, 3), ids, fat


def chains_with_load():
    """Joint chains with loose bodies falling onto them (contacts and joints in one island)."""
    rng = scenes.SplitMix64(3)
    s = scenes.chains(6, 16, rng)
    for k in range(24):
        x = -8.0 + 0.7 * k
        b = s.body(scenes.DYNAMIC, x, 22.0 + 0.3 * (k % 5))
        if k % 2:
            s.fixture(b, scenes.CIRCLE, [0.0, 0.0, 0.3], density=1.0, friction=0.4)
        else:
            s.fixture(b, scenes.BOX, [0.25, 0.25], 2, density=1.0, friction=0.4)
    return s


def run_case(scene, steps, checkpoints, kind, trig):
    w = oracle.OracleWorld(scene, kind, trig)
    digests = np.zeros((steps, 32), dtype=np.uint8)
    cps = {}
    for s in range(1, steps + 1):
        w.step(DT, VI, PI)
        b = w.bodies()
        ci, cf = w.contacts()
        digests[s - 1] = np.frombuffer(state_digest(b, ci, cf), dtype=np.uint8)
        if s in checkpoints:
            cps[f"bodies_{s}"] = b
            cps[f"cints_{s}"] = ci
            cps[f"cflts_{s}"] = cf
    return digests, cps


def random_shape(rng: scenes.SplitMix64, kind: int):
    """A shape in the C-ABI encoding: (type, shape list, n)."""
    if kind == 0:
        return 0, [rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3), rng.uniform(0.2, 1.0)], 0
    if kind == 1:
        x1, y1 = rng.uniform(-3, 3), rng.uniform(-1, 1)
        x2, y2 = rng.uniform(-3, 3), rng.uniform(-1, 1)
        has0, has3 = rng.randint(0, 1), rng.randint(0, 1)
        return 1, [x1, y1, x2, y2, x1 - rng.uniform(0.5, 2), y1 + rng.uniform(-1, 1), x2 + rng.uniform(0.5, 2),
                   y2 + rng.uniform(-1, 1), has0, has3], 0
    if kind == 2:
        k = rng.randint(3, 8)
        r = rng.uniform(0.3, 1.2)
        pts = []
        for i in range(k):
            a = 2 * math.pi * (i + rng.uniform(-0.3, 0.3)) / k
            pts += [round(r * math.cos(a) * 1048576) / 1048576, round(r * math.sin(a) * 1048576) / 1048576]
        return 2, pts, k
    return 3, [rng.uniform(0.2, 1.0), rng.uniform(0.2, 1.0)], 2


def xf_of(rng: scenes.SplitMix64, spread: float):
    a = rng.uniform(-math.pi, math.pi)
    s, c = oracle.sincosf("reference", "libm", a)
    return [rng.uniform(-spread, spread), rng.uniform(-spread, spread), s, c]


def make_collide(n: int = 4000):
    rng = scenes.SplitMix64(2024)
    pairs = [(0, 0), (2, 0), (3, 0), (2, 2), (3, 3), (2, 3), (1, 0), (1, 2), (1, 3)]
    ta, sa, na, xa, tb, sb, nb, xb, oi, of = [], [], [], [], [], [], [], [], [], []
    for k in range(n):
        ka, kb = pairs[k % len(pairs)]
        t1, s1, n1 = random_shape(rng, ka)
        t2, s2, n2 = random_shape(rng, kb)
        x1 = xf_of(rng, 0.2 if ka != 1 else 0.0)
        x2 = xf_of(rng, 1.2)
        i, f = oracle.collide("reference", "libm", t1, s1, n1, x1, t2, s2, n2, x2)
        pad = lambda s: list(s) + [0.0] * (16 - len(s))
        ta.append(t1); sa.append(pad(s1)); na.append(n1); xa.append(x1)
        tb.append(t2); sb.append(pad(s2)); nb.append(n2); xb.append(x2)
        oi.append(i); of.append(f)
    np.savez_compressed(os.path.join(HERE, "collide.npz"),
                        type_a=np.array(ta, np.int32), shape_a=np.array(sa, np.float32), n_a=np.array(na, np.int32),
                        xf_a=np.array(xa, np.float32), type_b=np.array(tb, np.int32), shape_b=np.array(sb, np.float32),
                        n_b=np.array(nb, np.int32), xf_b=np.array(xb, np.float32), out_ints=np.array(oi, np.int32),
                        out_floats=np.array(of, np.float32))


def make_toi(n: int = 1500):
    rng = scenes.SplitMix64(77)
    rows, outs = [], []
    for k in range(n):
        ta, sa, na = random_shape(rng, [0, 2, 3][k % 3])
        tb, sb, nb = random_shape(rng, [0, 2, 3][(k // 3) % 3])
        c0 = [rng.uniform(-0.5, 0.5), rng.uniform(2.0, 4.0)]
        c = [c0[0] + rng.uniform(-1, 1), c0[1] - rng.uniform(1.0, 5.0)]
        swa = [0.0, 0.0, c0[0], c0[1], c[0], c[1], rng.uniform(-1, 1), rng.uniform(-2, 2), 0.0]
        swb = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
        st, t = oracle.toi("reference", "project", ta, sa, na, swa, tb, sb, nb, swb)
        pad = lambda s: list(s) + [0.0] * (16 - len(s))
        rows.append((ta, pad(sa), na, swa, tb, pad(sb), nb, swb))
        outs.append((st, t))
    np.savez_compressed(os.path.join(HERE, "toi.npz"),
                        type_a=np.array([r[0] for r in rows], np.int32), shape_a=np.array([r[1] for r in rows], np.float32),
                        n_a=np.array([r[2] for r in rows], np.int32), sweep_a=np.array([r[3] for r in rows], np.float32),
                        type_b=np.array([r[4] for r in rows], np.int32), shape_b=np.array([r[5] for r in rows], np.float32),
                        n_b=np.array([r[6] for r in rows], np.int32), sweep_b=np.array([r[7] for r in rows], np.float32),
                        state=np.array([o[0] for o in outs], np.int32), t=np.array([o[1] for o in outs], np.float32))


def query_scenes():
    """Scenes the world-query golden vectors are taken on, with the steps run before the queries."""
    return [
        ("drop300", lambda: scenes.drop(300, scenes.SplitMix64(7)), 90),
        ("pyramid20", lambda: scenes.config1(), 60),
        ("chains", lambda: chains_with_load(), 60),
        ("batch3", lambda: batch_world(3), 60),
    ]


def make_queries(n_boxes: int = 300, n_rays: int = 600):
    """b2World::QueryAABB and closest-hit b2World::RayCast results of the reference (project trig) on
    stepped scenes, for seeded boxes and segments over each scene's extent."""
    out = {}
    for name, make, steps in query_scenes():
        sc = make()
        w = oracle.OracleWorld(sc, "reference", "project")
        for _ in range(steps):
            w.step(DT, VI, PI)
        b = w.bodies()
        lo, hi = b[:, 0:2].min(axis=0) - 2.0, b[:, 0:2].max(axis=0) + 2.0
        rng = scenes.SplitMix64(zlib.crc32(name.encode()))
        boxes, rays = [], []
        for _ in range(n_boxes):
            cx, cy = rng.uniform(lo[0], hi[0]), rng.uniform(lo[1], hi[1])
            hx, hy = rng.uniform(0.1, 6.0), rng.uniform(0.1, 6.0)
            boxes.append([cx - hx, cy - hy, cx + hx, cy + hy])
        for _ in range(n_rays):
            rays.append([rng.uniform(lo[0], hi[0]), rng.uniform(lo[1], hi[1]), rng.uniform(lo[0], hi[0]),
                         rng.uniform(lo[1], hi[1])])
        boxes = np.array(boxes, dtype=np.float32)
        rays = np.array(rays, dtype=np.float32)
        counts, fixtures = [], []
        for bx in boxes:
            f = w.query_aabb(bx)
            counts.append(len(f))
            fixtures.extend(f.tolist())
        ray_fix, ray_hit = [], []
        for r in rays:
            f, h = w.raycast(r)
            ray_fix.append(f)
            ray_hit.append(h)
        out[name] = dict(boxes=boxes, counts=np.array(counts, np.int32), fixtures=np.array(fixtures, np.int32),
                         rays=rays, ray_fixture=np.array(ray_fix, np.int32), ray_hit=np.array(ray_hit, np.float32),
                         steps=np.int32(steps))
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, f"query_{name}.npz"), **d)


def make_trig(n: int = 200000):
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(-4, 4, n // 2), rng.uniform(-1e-3, 1e-3, n // 4),
                        rng.uniform(-200, 200, n // 4)]).astype(np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    for i, v in enumerate(x):
        s[i], c[i] = oracle.sincosf("reference", "libm", float(v))
    np.savez_compressed(os.path.join(HERE, "trig.npz"), x=x, sin=s, cos=c)


def tree_cases():
    """Cases of tree_stats.npz: (name, scene factory, steps, ops by step)."""
    from tests._util import body_props_script, destroy_script, fixture_props_script, shift_script

    return [("pyramid20", lambda: scenes.config1(), 200, {}),
            ("drop300", lambda: scenes.drop(300, scenes.SplitMix64(7)), 300, {}),
            ("chains6x16", lambda: chains_with_load(), 200, {}),
            ("chain_terrain", lambda: scenes.chain_terrain(scenes.SplitMix64(12)), 200, {}),
            ("sensors", lambda: scenes.sensors(scenes.SplitMix64(13)), 200, {}),
            ("batch3", lambda: batch_world(3), 200, {}),
            ("config2_10k", lambda: scenes.config2(10000, seed=1, allow_sleep=True), 100, {}),
            ("destroy_mix", lambda: scenes.destroy_mix(scenes.SplitMix64(5)), 200, destroy_script()),
            ("body_props", lambda: scenes.destroy_mix(scenes.SplitMix64(11)), 320, body_props_script()),
            ("fixture_props", lambda: scenes.destroy_mix(scenes.SplitMix64(13)), 300, fixture_props_script()),
            ("shift_origin", lambda: scenes.pulley_mouse(scenes.SplitMix64(4)), 260, shift_script())]


def make_tree():
    """b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality of the reference (project trig) after
    every step: ``<case>_hb`` (steps x 2 int32, height and balance), ``<case>_quality`` (float32)."""
    from tests._util import apply_ops

    out = {}
    for name, make, steps, script in tree_cases():
        w = oracle.OracleWorld(make(), "reference", "project")
        hb = np.zeros((steps, 2), dtype=np.int32)
        q = np.zeros(steps, dtype=np.float32)
        for s in range(1, steps + 1):
            if s in script:
                apply_ops(w, script[s])
            w.step(DT, VI, PI)
            h, b, qq = w.tree_stats()
            hb[s - 1] = (h, b)
            q[s - 1] = qq
        out[f"{name}_hb"] = hb
        out[f"{name}_quality"] = q
    np.savez_compressed(os.path.join(HERE, "tree_stats.npz"), **out)


def fixture_query_inputs(bodies: np.ndarray, fix_body: np.ndarray, seed: int = 3):
    """Seeded b2Fixture queries around each fixture's body: rows (fixture, op, 5 inputs); op 0 a point
    within 1 m of the body origin, op 1 a 6 m horizontal-ish ray through it (maxFraction 1), op 2 the
    box."""
    rng = np.random.default_rng(seed)
    rows = []
    for f, b in enumerate(fix_body):
        px, py = float(bodies[b, 0]), float(bodies[b, 1])
        for _ in range(4):
            rows.append([f, 0, px + rng.uniform(-1, 1), py + rng.uniform(-1, 1), 0.0, 0.0, 0.0])
            rows.append([f, 1, px - 3.0, py + rng.uniform(-0.5, 0.5), px + 3.0, py + rng.uniform(-0.5, 0.5), 1.0])
        rows.append([f, 2, 0.0, 0.0, 0.0, 0.0, 0.0])
    return np.array(rows, dtype=np.float32)


def make_fixture_queries(steps: int = 60):
    """b2Fixture::TestPoint, RayCast and GetAABB of every fixture of destroy_mix (seed 5) after `steps`
    steps of the reference (project trig): inputs (fixture, op, 5 floats) and outputs (4 floats)."""
    sc = scenes.destroy_mix(scenes.SplitMix64(5))
    w = oracle.OracleWorld(sc, "reference", "project")
    for _ in range(steps):
        w.step(DT, VI, PI)
    q = fixture_query_inputs(w.bodies(), sc.arrays()["fix_body"])
    out = np.array([w.fixture_query(int(r[0]), int(r[1]), r[2:]) for r in q], dtype=np.float32)
    np.savez_compressed(os.path.join(HERE, "fixture_queries.npz"), queries=q, outputs=out, steps=np.int32(steps))


def main():
    oracle.build_reference()
    if "--fixture-queries" in sys.argv:
        make_fixture_queries()
        print("done")
        return
    if "--queries" in sys.argv:
        make_queries()
        print("done")
        return
    if "--tree" in sys.argv:
        make_tree()
        print("done")
        return
    only = sys.argv[sys.argv.index("--case") + 1] if "--case" in sys.argv else None
    if only in (None, "presolve_rule"):
        from tests._util import presolve_case

        sc, bits = presolve_case()
        for trig in ("libm", "project"):
            w = oracle.OracleWorld(sc, "reference", trig)
            w.set_presolve_rule(bits)
            digests = np.zeros((300, 32), dtype=np.uint8)
            for s in range(1, 301):
                w.step(DT, VI, PI)
                digests[s - 1] = np.frombuffer(state_digest(w.bodies(), *w.contacts()), dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, f"presolve_rule_{trig}.npz"), digests=digests, steps=np.int32(300))
        print("wrote presolve_rule")
    if only in (None, "filter_rule"):
        sc = scenes.drop(200, scenes.SplitMix64(29))
        for trig in ("libm", "project"):
            w = oracle.OracleWorld(sc, "reference", trig)
            w.set_filter_rule(5, 4)
            digests = np.zeros((300, 32), dtype=np.uint8)
            for s in range(1, 301):
                w.step(DT, VI, PI)
                digests[s - 1] = np.frombuffer(state_digest(w.bodies(), *w.contacts()), dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, f"filter_rule_{trig}.npz"), digests=digests, steps=np.int32(300))
        print("wrote filter_rule")
    for name, make, steps, script in scripted_cases():
        if only and name != only:
            continue
        for trig in ("libm", "project"):
            digests, calls, ids, fat = run_scripted(make(), steps, script, trig)
            np.savez_compressed(os.path.join(HERE, f"{name}_{trig}.npz"), digests=digests, goodbyes=calls,
                                proxy_ids=ids, proxy_fat=fat, steps=np.int32(steps))
        print("wrote", name)
    for name, make, steps, cps in cases():
        if only and name != only:
            continue
        for trig in ("libm", "project"):
            digests, snap = run_case(make(), steps, cps, "reference", trig)
            np.savez_compressed(os.path.join(HERE, f"{name}_{trig}.npz"), digests=digests,
                                checkpoints=np.array(cps, np.int32), steps=np.int32(steps), **snap)
        print("wrote", name)
    if only:
        return
    make_collide()
    make_toi()
    make_trig()
    make_queries()
    make_tree()
    make_fixture_queries()
    print("done")


if __name__ == "__main__":
    main()
