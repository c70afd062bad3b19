"""Python handle over the GB300 step: one ``World`` owns a batch of independent Box2D worlds.

Built from ``scenes.Scene`` descriptions (the calls a b2World user makes), stepped on the GPU through
the C-ABI, and read back in the same layouts the oracle uses so the two compare directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .scenes import Scene


class World:
    """A batch of Box2D worlds resident on the GPU (a single world is a batch of one)."""

    def __init__(self, scenes, track_tree: bool = False):
        """track_tree: keep every world's broadphase tree on the host for tree_stats (see
        gb_world_track_tree; each step then waits for the previous one)."""
        if isinstance(scenes, Scene):
            scenes = [scenes]
        self.lib = _lib.load()
        self.n_worlds = len(scenes)
        defs = (_lib.WorldDef * self.n_worlds)()
        for i, s in enumerate(scenes):
            defs[i].gravity_x, defs[i].gravity_y = float(s.gravity[0]), float(s.gravity[1])
            defs[i].allow_sleep, defs[i].warm_starting = int(s.allow_sleep), int(s.warm_starting)
            defs[i].continuous_physics, defs[i].sub_stepping = int(s.continuous), int(s.sub_stepping)
        h = C.c_void_p()
        _lib.check(self.lib.gb_world_create(self.n_worlds, defs, C.byref(h)), "gb_world_create")
        self.h = h
        if track_tree:
            _lib.check(self.lib.gb_world_track_tree(self.h, 1), "gb_world_track_tree")
        self.n_fixtures = []
        self.n_bodies = []
        self.dynamic_bodies = 0
        for i, s in enumerate(scenes):
            a = s.arrays()
            _lib.check(self.lib.gb_build_world(
                self.h, i, len(a["body_type"]), a["body_type"], a["body_f"], a["body_flags"], len(a["fix_body"]),
                a["fix_body"], a["fix_type"], a["fix_shape"], a["fix_n"], a["fix_mat"], a["fix_filt"],
                len(a["joint_a"]), a["joint_type"], a["joint_a"], a["joint_b"], a["joint_f"], a["joint_flags"]),
                "gb_build_world")
            self.n_fixtures.append(len(a["fix_body"]))
            self.n_bodies.append(len(a["body_type"]))
            self.dynamic_bodies += int((a["body_type"] == 2).sum())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gb_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ stepping
    def upload(self) -> None:
        _lib.check(self.lib.gb_world_upload(self.h), "gb_world_upload")

    def step(self, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> None:
        _lib.check(self.lib.gb_world_step(self.h, dt, vi, pi), "gb_world_step")

    def set_contact_filter(self, should_collide=None) -> None:
        """b2World::SetContactFilter: should_collide(world, fixtureA, fixtureB) -> bool, or None for
        the default filter (see gb_world_set_contact_filter)."""
        if should_collide is None:
            self._filter_cb = None
            _lib.check(self.lib.gb_world_set_contact_filter(self.h, _lib.SHOULD_COLLIDE_FN(), None),
                       "gb_world_set_contact_filter")
            return
        self._filter_cb = _lib.SHOULD_COLLIDE_FN(lambda _u, w, a, b: 1 if should_collide(w, a, b) else 0)
        _lib.check(self.lib.gb_world_set_contact_filter(self.h, self._filter_cb, None), "gb_world_set_contact_filter")

    def filter_stats(self):
        """(steps run again, verdicts kept) of the user contact filter."""
        r, v = C.c_longlong(), C.c_int()
        _lib.check(self.lib.gb_world_filter_stats(self.h, C.byref(r), C.byref(v)), "gb_world_filter_stats")
        return r.value, v.value

    def step_begin(self, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> None:
        """First half of a split step: up to and including the collide phase (gb_world_step_begin)."""
        _lib.check(self.lib.gb_world_step_begin(self.h, dt, vi, pi), "gb_world_step_begin")

    def contact_edits(self, edits) -> None:
        """Contact changes between the halves: (world, list position, flags, enabled, friction,
        restitution, tangent speed) records (see gb_contact_edits)."""
        arr = np.zeros(len(edits), dtype=_lib.CONTACT_EDIT_DTYPE)
        for k, e in enumerate(edits):
            arr[k] = tuple(e) + (0.0,) * (8 - len(e))
        _lib.check(self.lib.gb_contact_edits(self.h, len(arr), arr.ctypes.data if len(arr) else None),
                   "gb_contact_edits")

    def step_end(self) -> None:
        """Second half of a split step (gb_world_step_end)."""
        _lib.check(self.lib.gb_world_step_end(self.h), "gb_world_step_end")

    def graph_step(self, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> None:
        """One step replayed from a captured CUDA graph (see gb_world_graph_step)."""
        _lib.check(self.lib.gb_world_graph_step(self.h, dt, vi, pi), "gb_world_graph_step")

    def sync(self) -> None:
        _lib.check(self.lib.gb_world_sync(self.h), "gb_world_sync")

    def set_solver(self, solver: str = "plain", tolerance: float = 0.0, measure_residual: bool = False) -> None:
        """Island solver of the following steps: "plain" (the reference's sequential order, bit-exact)
        or "coloured" (parallel per constraint colour); see gb_world_set_solver."""
        code = {"plain": _lib.SOLVER_PLAIN, "coloured": _lib.SOLVER_COLOURED}[solver]
        _lib.check(self.lib.gb_world_set_solver(self.h, code, float(tolerance), int(measure_residual)),
                   "gb_world_set_solver")

    # ------------------------------------------------------------------ changes between steps
    def add_body(self, type_: int, f, flags: int, w: int = 0) -> int:
        """b2World::CreateBody between steps (f: the 9 floats of the body encoding); returns its index."""
        out = np.zeros(1, dtype=np.int32)
        _lib.check(self.lib.gb_create_bodies(self.h, w, 1, np.array([type_], np.int32),
                                             np.ascontiguousarray(f, dtype=np.float32), np.array([flags], np.int32),
                                             out), "gb_create_bodies")
        self.n_bodies[w] += 1
        if type_ == 2:
            self.dynamic_bodies += 1
        return int(out[0])

    def add_fixture(self, body: int, type_: int, shape, n: int, mat, filt, w: int = 0) -> int:
        """b2Body::CreateFixture between steps (one fixture record); returns its index."""
        s = np.zeros(16, dtype=np.float32)
        s[:len(shape)] = shape
        out = np.zeros(1, dtype=np.int32)
        _lib.check(self.lib.gb_create_fixtures(self.h, w, 1, np.array([body], np.int32), np.array([type_], np.int32),
                                               s, np.array([n], np.int32), np.asarray(mat, dtype=np.float32),
                                               np.asarray(filt, dtype=np.int32), out), "gb_create_fixtures")
        self.n_fixtures[w] += 1
        return int(out[0])

    def _destroy(self, fn: str, index: int, w: int):
        calls = np.zeros((256, 3), dtype=np.int32)
        n = C.c_int()
        _lib.check(getattr(self.lib, fn)(self.h, w, int(index), calls, 256, C.byref(n)), fn)
        return calls[:min(n.value, 256)]

    def destroy_body(self, body: int, w: int = 0) -> np.ndarray:
        """b2World::DestroyBody; returns the listener calls as rows {kind, a, b} (see gb_destroy_body):
        kind 0 SayGoodbye(joint a), 1 SayGoodbye(fixture a), 2 EndContact(a, b)."""
        return self._destroy("gb_destroy_body", body, w)

    def checkpoint(self, w: int = 0) -> bytes:
        """World w's whole state between steps (gb_world_checkpoint), as bytes."""
        n = C.c_size_t()
        _lib.check(self.lib.gb_world_checkpoint(self.h, int(w), None, 0, C.byref(n)), "gb_world_checkpoint")
        buf = C.create_string_buffer(n.value)
        _lib.check(self.lib.gb_world_checkpoint(self.h, int(w), buf, n.value, C.byref(n)), "gb_world_checkpoint")
        return buf.raw[:n.value]

    def restore(self, data: bytes, w: int = 0) -> None:
        """Replaces world w with a checkpoint (gb_world_restore); the following steps are those of the
        world it was taken from, bit for bit."""
        _lib.check(self.lib.gb_world_restore(self.h, int(w), data, len(data)), "gb_world_restore")
        b, f, c, j = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(self.lib.gb_world_counts(self.h, int(w), C.byref(b), C.byref(f), C.byref(c), C.byref(j)),
                   "gb_world_counts")
        self.n_bodies[w], self.n_fixtures[w] = b.value, f.value

    def tree_stats(self, w: int = 0):
        """b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality of world w: (height, balance,
        quality); the handle must have been made with track_tree=True."""
        h, b, q = C.c_int(), C.c_int(), C.c_float()
        _lib.check(self.lib.gb_world_tree_stats(self.h, int(w), C.byref(h), C.byref(b), C.byref(q)),
                   "gb_world_tree_stats")
        return h.value, b.value, np.float32(q.value)

    def body_set(self, body: int, prop: int, value=0.0, w: int = 0) -> np.ndarray:
        """b2Body::SetType (prop BODY_TYPE, value 0 static / 1 kinematic / 2 dynamic), SetActive,
        SetFixedRotation, SetBullet, SetSleepingAllowed (flags: value != 0), SetLinearDamping,
        SetAngularDamping, SetGravityScale, SetMassData (value = mass, center x, center y, inertia)
        or ResetMassData between steps; returns the EndContact calls of the contacts it destroys as
        rows {2, fixtureA, fixtureB}."""
        calls = np.zeros((256, 3), dtype=np.int32)
        n = C.c_int()
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        _lib.check(self.lib.gb_body_set(self.h, int(w), int(body), int(prop), v, calls, 256, C.byref(n)),
                   "gb_body_set")
        return calls[:min(n.value, 256)]

    def fixture_query(self, fixture: int, op: int, inp=(), w: int = 0) -> np.ndarray:
        """b2Fixture::TestPoint (op 0), RayCast (op 1: p1, p2, maxFraction -> hit, normal, fraction),
        GetAABB (op 2) or GetMassData (op 3: mass, center, inertia) at the body's current transform
        (gb_fixture_query), as float32."""
        v = np.zeros(8, dtype=np.float32)
        v[:len(inp)] = inp
        out = np.zeros(4, dtype=np.float32)
        _lib.check(self.lib.gb_fixture_query(self.h, int(w), int(fixture), int(op), v, out), "gb_fixture_query")
        return out

    def joint_reaction(self, joint: int, inv_dt: float, w: int = 0) -> np.ndarray:
        """b2Joint::GetReactionForce and GetReactionTorque after the last step: (force x, force y,
        torque) as float32 (gb_get_joint_reaction)."""
        out = np.zeros(3, dtype=np.float32)
        _lib.check(self.lib.gb_get_joint_reaction(self.h, int(w), int(joint), float(inv_dt), out),
                   "gb_get_joint_reaction")
        return out

    def joint_set(self, joint: int, prop: int, value=0.0, w: int = 0) -> None:
        """A joint setter between steps (gb_joint_set; prop GB_JOINT_*, value a number or a pair)."""
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        _lib.check(self.lib.gb_joint_set(self.h, int(w), int(joint), int(prop), v), "gb_joint_set")

    def shift_origin(self, x: float, y: float, w: int = 0) -> None:
        """b2World::ShiftOrigin(b2Vec2(x, y)) of world w between steps."""
        _lib.check(self.lib.gb_world_shift_origin(self.h, int(w), float(x), float(y)), "gb_world_shift_origin")

    def fixture_set(self, fixture: int, prop: int, value=0.0, w: int = 0) -> np.ndarray:
        """b2Fixture::SetFriction, SetRestitution, SetDensity, SetSensor or SetFilterData (value =
        category, mask, group) between steps (gb_fixture_set); makes no listener calls."""
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        _lib.check(self.lib.gb_fixture_set(self.h, int(w), int(fixture), int(prop), v), "gb_fixture_set")
        return np.zeros((0, 3), dtype=np.int32)

    def body_info(self, body: int, w: int = 0):
        """(mass, inertia, local center x, y, linear damping, angular damping, gravity scale) as float32
        and the flags (type | 4 bullet | 8 fixed rotation | 16 sleeping allowed | 32 active) of a body
        (gb_get_body_info)."""
        out = np.zeros(7, dtype=np.float32)
        fl = C.c_int()
        _lib.check(self.lib.gb_get_body_info(self.h, int(w), int(body), out, C.byref(fl)), "gb_get_body_info")
        return out, fl.value

    def destroy_joint(self, joint: int, w: int = 0) -> np.ndarray:
        """b2World::DestroyJoint (no listener calls)."""
        return self._destroy("gb_destroy_joint", joint, w)

    def destroy_fixture(self, fixture: int, w: int = 0) -> np.ndarray:
        """b2Body::DestroyFixture; returns its EndContact calls as rows {2, fixtureA, fixtureB}."""
        return self._destroy("gb_destroy_fixture", fixture, w)

    def set_settings(self, gravity, allow_sleep: bool, warm_starting: bool, continuous: bool, sub_stepping: bool,
                     auto_clear_forces: bool = True, w: int = 0) -> None:
        """b2World::SetGravity, SetAllowSleeping (turning it off wakes every body), SetWarmStarting,
        SetContinuousPhysics, SetSubStepping and SetAutoClearForces of world w between steps."""
        d = _lib.WorldDef()
        d.gravity_x, d.gravity_y = float(gravity[0]), float(gravity[1])
        d.allow_sleep, d.warm_starting = int(allow_sleep), int(warm_starting)
        d.continuous_physics, d.sub_stepping = int(continuous), int(sub_stepping)
        _lib.check(self.lib.gb_world_set_settings(self.h, int(w), C.byref(d), int(auto_clear_forces)),
                   "gb_world_set_settings")

    def clear_forces(self, w: int = 0) -> None:
        """b2World::ClearForces of world w."""
        _lib.check(self.lib.gb_world_clear_forces(self.h, int(w)), "gb_world_clear_forces")

    def set_recovery(self, attempts: int) -> None:
        """Grow-and-retry of overflowing steps (gb_world_set_recovery); 0 turns it off."""
        _lib.check(self.lib.gb_world_set_recovery(self.h, int(attempts)), "gb_world_set_recovery")

    def recoveries(self) -> int:
        """Steps run again after an overflow so far."""
        n = C.c_longlong()
        _lib.check(self.lib.gb_world_recoveries(self.h, C.byref(n)), "gb_world_recoveries")
        return n.value

    def set_limits(self, contact_capacity: int = 0, max_toi_events: int = 4096) -> None:
        """Fixed capacities of the device step (see gb_world_set_limits): contact slots per world at
        the first upload (0: the default) and time-of-impact events per world per step."""
        _lib.check(self.lib.gb_world_set_limits(self.h, int(contact_capacity), int(max_toi_events)),
                   "gb_world_set_limits")

    def solver_stats(self):
        """(colours, velocity iterations, velocity residual) per world of the last step."""
        col = np.zeros(self.n_worlds, dtype=np.int32)
        its = np.zeros(self.n_worlds, dtype=np.int32)
        res = np.zeros(self.n_worlds, dtype=np.float32)
        _lib.check(self.lib.gb_world_solver_stats(self.h, col, its, res), "gb_world_solver_stats")
        return col, its, res

    def autotune(self, steps_per_candidate: int = 2) -> None:
        """Arm the online launch-plan autotuner over the next steps (see gb_world_autotune)."""
        _lib.check(self.lib.gb_world_autotune(self.h, int(steps_per_candidate)), "gb_world_autotune")

    def launch_plan(self):
        """(classes as rows of first, count, threads, smem rows, smem contacts; best ms per candidate)."""
        cls = np.zeros(5 * 8, dtype=np.int32)
        ms = np.zeros(32, dtype=np.float32)
        n, nc = C.c_int(), C.c_int()
        _lib.check(self.lib.gb_world_launch_plan(self.h, cls, 8, C.byref(n), ms, 32, C.byref(nc)),
                   "gb_world_launch_plan")
        return cls[:5 * n.value].reshape(n.value, 5), ms[:nc.value]

    def set_launch_plan(self, classes) -> None:
        arr = np.ascontiguousarray(np.asarray(classes, dtype=np.int32).reshape(-1, 5))
        _lib.check(self.lib.gb_world_set_launch_plan(self.h, arr.reshape(-1), len(arr)), "gb_world_set_launch_plan")

    def set_warm_start(self, mlp=None, all_points: bool = False) -> None:
        """Learned warm start with the given network (reference warm start as fallback); None: the
        reference warm start only. all_points: the network corrects every contact point, not only
        the ones the reference starts cold. The network must outlive its use by this world."""
        if mlp is None:
            _lib.check(self.lib.gb_world_set_warm_start(self.h, None, _lib.WARM_REFERENCE), "gb_world_set_warm_start")
        else:
            mode = _lib.WARM_LEARNED_ALL if all_points else _lib.WARM_LEARNED
            _lib.check(self.lib.gb_world_set_warm_start(self.h, mlp.h, mode), "gb_world_set_warm_start")
        self._mlp = mlp

    def warm_stats(self):
        """(islands that kept the learned warm start, velocity iterations summed over islands) per world."""
        used = np.zeros(self.n_worlds, dtype=np.int32)
        its = np.zeros(self.n_worlds, dtype=np.int32)
        _lib.check(self.lib.gb_world_warm_stats(self.h, used, its), "gb_world_warm_stats")
        return used, its

    def set_contact_log(self, capacity: int) -> None:
        _lib.check(self.lib.gb_world_set_contact_log(self.h, int(capacity)), "gb_world_set_contact_log")
        self._log_cap = int(capacity)

    def read_contact_log(self):
        """(features [n][14], targets [n][2]) logged since the last read; empties the log."""
        cap = getattr(self, "_log_cap", 0)
        x = np.zeros((max(cap, 1), 14), dtype=np.float32)
        t = np.zeros((max(cap, 1), 2), dtype=np.float32)
        n = C.c_int()
        _lib.check(self.lib.gb_world_read_contact_log(self.h, x, t, cap, C.byref(n)), "gb_world_read_contact_log")
        return x[:n.value], t[:n.value]

    def max_penetration(self) -> np.ndarray:
        """Per world: the deepest penetration (m) the last step's position solver started from."""
        out = np.zeros(self.n_worlds, dtype=np.float32)
        _lib.check(self.lib.gb_world_contact_stats(self.h, out), "gb_world_contact_stats")
        return out

    def set_events(self, on: bool = True) -> None:
        """Record the listener calls of every step on the device (see gb_world_set_events)."""
        _lib.check(self.lib.gb_world_set_events(self.h, int(on)), "gb_world_set_events")

    def events(self, w: int = 0):
        """(records [n][4] = kind, fixtureA, fixtureB, impulse points; impulses [n][4] = n0, n1, t0, t1) of
        the last step."""
        n = C.c_int()
        _lib.check(self.lib.gb_world_read_events(self.h, w, np.zeros(4, np.int32), np.zeros(4, np.float32), 0,
                                                 C.byref(n)), "gb_world_read_events")
        cnt = n.value
        rec = np.zeros((max(cnt, 1), 4), dtype=np.int32)
        imp = np.zeros((max(cnt, 1), 4), dtype=np.float32)
        _lib.check(self.lib.gb_world_read_events(self.h, w, rec, imp, cnt, C.byref(n)), "gb_world_read_events")
        return rec[:cnt], imp[:cnt]

    def query_aabb(self, boxes, w: int = 0):
        """Fixture indices whose fat AABB overlaps each box (lower.x, lower.y, upper.x, upper.y): a list
        of arrays, one per box (see gb_world_query_aabb)."""
        boxes = np.ascontiguousarray(np.asarray(boxes, dtype=np.float32).reshape(-1, 4))
        n = len(boxes)
        offsets = np.zeros(n + 1, dtype=np.int32)
        total = C.c_int()
        status = self.lib.gb_world_query_aabb(self.h, w, n, boxes, offsets, np.zeros(1, np.int32), 0, C.byref(total))
        if status not in (_lib.GB_OK, _lib.GB_ERR_CAPACITY):
            _lib.check(status, "gb_world_query_aabb")
        fixtures = np.zeros(max(total.value, 1), dtype=np.int32)
        _lib.check(self.lib.gb_world_query_aabb(self.h, w, n, boxes, offsets, fixtures, total.value, C.byref(total)),
                   "gb_world_query_aabb")
        return [fixtures[offsets[i]:offsets[i + 1]].copy() for i in range(n)]

    def raycast(self, rays, w: int = 0):
        """Closest hit per segment (p1.x, p1.y, p2.x, p2.y): (fixture or -1, [fraction, point.x, point.y,
        normal.x, normal.y]) arrays (see gb_world_raycast)."""
        rays = np.ascontiguousarray(np.asarray(rays, dtype=np.float32).reshape(-1, 4))
        n = len(rays)
        fixture = np.zeros(max(n, 1), dtype=np.int32)
        hit = np.zeros((max(n, 1), 5), dtype=np.float32)
        _lib.check(self.lib.gb_world_raycast(self.h, w, n, rays, fixture, hit), "gb_world_raycast")
        return fixture[:n], hit[:n]

    def raycast_all(self, ray, w: int = 0):
        """Every fixture the segment hits (gb_world_raycast_all): (fixtures, hits[k] = fraction, point,
        normal), in fixture order."""
        nf = self.n_fixtures[w]
        fix = np.zeros(max(nf, 1), dtype=np.int32)
        hits = np.zeros((max(nf, 1), 5), dtype=np.float32)
        n = C.c_int()
        _lib.check(self.lib.gb_world_raycast_all(self.h, w, np.ascontiguousarray(ray, dtype=np.float32), fix, hits,
                                                 nf, C.byref(n)), "gb_world_raycast_all")
        return fix[:n.value], hits[:n.value]

    def profile_ms(self, w: int = 0) -> dict:
        """b2World::GetProfile of the last step (gb_world_get_profile), milliseconds."""
        out = np.zeros(8, dtype=np.float32)
        _lib.check(self.lib.gb_world_get_profile(self.h, w, out), "gb_world_get_profile")
        keys = ["step", "collide", "solve", "solveInit", "solveVelocity", "solvePosition", "broadphase", "solveTOI"]
        return dict(zip(keys, map(float, out)))

    def set_stream(self, stream_handle: int) -> None:
        _lib.check(self.lib.gb_world_set_stream(self.h, C.c_void_p(stream_handle)), "gb_world_set_stream")

    # ------------------------------------------------------------------ read-back
    def counts(self, w: int = 0):
        b, f, c, j = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(self.lib.gb_world_counts(self.h, w, C.byref(b), C.byref(f), C.byref(c), C.byref(j)), "gb_world_counts")
        return b.value, f.value, c.value, j.value

    def bodies(self, w: int = 0) -> np.ndarray:
        out = np.zeros((max(self.n_bodies[w], 1), 12), dtype=np.float32)
        _lib.check(self.lib.gb_get_bodies(self.h, w, out), "gb_get_bodies")
        return out[:self.n_bodies[w]]

    def contacts(self, w: int = 0):
        n = C.c_int()
        probe_i, probe_f = np.zeros((1, 8), dtype=np.int32), np.zeros((1, 12), dtype=np.float32)
        _lib.check(self.lib.gb_get_contacts(self.h, w, probe_i, probe_f, 0, C.byref(n)), "gb_get_contacts")
        cnt = n.value
        ints = np.zeros((max(cnt, 1), 8), dtype=np.int32)
        flts = np.zeros((max(cnt, 1), 12), dtype=np.float32)
        _lib.check(self.lib.gb_get_contacts(self.h, w, ints, flts, cnt, C.byref(n)), "gb_get_contacts")
        return ints[:cnt], flts[:cnt]

    def proxies(self, w: int = 0):
        # sized from the library's count: fixtures may have been added by direct C-ABI calls
        n = C.c_int()
        _lib.check(self.lib.gb_world_counts(self.h, w, None, C.byref(n), None, None), "gb_world_counts")
        nf = n.value
        ids = np.zeros(max(nf, 1), dtype=np.int32)
        fat = np.zeros((max(nf, 1), 4), dtype=np.float32)
        _lib.check(self.lib.gb_get_proxies(self.h, w, ids, fat), "gb_get_proxies")
        return ids[:nf], fat[:nf]

    def stats(self, w: int = 0):
        isl, toi = C.c_int(), C.c_int()
        _lib.check(self.lib.gb_world_stats(self.h, w, C.byref(isl), C.byref(toi)), "gb_world_stats")
        return isl.value, toi.value

    def totals(self) -> dict:
        out = (C.c_longlong * 8)()
        _lib.check(self.lib.gb_world_totals(self.h, out), "gb_world_totals")
        keys = ["contacts", "solved_bodies", "solved_contacts", "pairs", "islands", "toi_events", "proxies",
                "dynamic_bodies"]
        return dict(zip(keys, list(out)))

    PHASES = ["new_pairs", "collide", "island_build", "island_solve", "fixture_sync", "pairs", "toi", "step",
              "solve_init", "solve_velocity", "solve_store_integrate", "solve_position", "solve_writeback",
              "solve_sleep", "pairs_find_sort", "pairs_create", "toi_classify", "toi_select", "toi_island",
              "toi_solve", "toi_sync", "toi_pairs", "build_components", "build_sort"]

    def profile(self) -> np.ndarray:
        """SM clock cycles per world and phase of the last step, shape (worlds, 24) (see PHASES)."""
        out = np.zeros(len(self.PHASES) * self.n_worlds, dtype=np.uint64)
        _lib.check(self.lib.gb_world_profile(self.h, out), "gb_world_profile")
        return out.reshape(self.n_worlds, len(self.PHASES))

    def body_edits(self, edits) -> None:
        """b2Body state changes before the next step, in order: edits is a sequence of (world, body,
        op name or code, values, wake) with op names from _lib.EDIT_OPS (see gb_body_edits); for
        "mouse_target" the body field is the mouse joint's index and values the new world target."""
        arr = np.zeros(len(edits), dtype=_lib.EDIT_DTYPE)
        for i, (w, b, op, vals, wake) in enumerate(edits):
            arr[i]["world"], arr[i]["body"] = w, b
            arr[i]["op"] = _lib.EDIT_OPS[op] if isinstance(op, str) else int(op)
            arr[i]["wake"] = int(bool(wake))
            v = np.zeros(4, dtype=np.float32)
            v[:len(vals)] = vals
            arr[i]["v"] = v
        _lib.check(self.lib.gb_body_edits(self.h, len(arr), arr.ctypes.data_as(C.c_void_p)), "gb_body_edits")

    STAGES = ["narrowphase_prepass", "step", "toi_prepass", "continuous"]

    def stage_times(self, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> np.ndarray:
        """Milliseconds of the four launch stages of one (real) step, see STAGES and gb_world_stage_times."""
        out = np.zeros(4, dtype=np.float32)
        _lib.check(self.lib.gb_world_stage_times(self.h, float(dt), int(vi), int(pi), out), "gb_world_stage_times")
        return out

    @property
    def total_bodies(self) -> int:
        return int(sum(self.n_bodies))

    def set_forces_ptr(self, host_ptr: int) -> None:
        """Queue an upload of force/torque (float4 per body, all worlds) from a host pointer."""
        _lib.check(self.lib.gb_set_forces(self.h, C.c_void_p(host_ptr)), "gb_set_forces")

    def get_transforms_ptr(self, host_ptr: int) -> None:
        """Copy every body transform (float4 per body, all worlds) into a host pointer."""
        _lib.check(self.lib.gb_get_transforms(self.h, C.c_void_p(host_ptr)), "gb_get_transforms")

    def set_forces_async_ptr(self, host_ptr: int) -> None:
        """Pipelined upload of force/torque (see gb_set_forces_async); the host memory must stay
        untouched until sync()."""
        _lib.check(self.lib.gb_set_forces_async(self.h, C.c_void_p(host_ptr)), "gb_set_forces_async")

    def get_transforms_async_ptr(self, host_ptr: int) -> None:
        """Pipelined read-back of every body transform after the queued steps (see
        gb_get_transforms_async); the host memory holds them once sync() returns."""
        _lib.check(self.lib.gb_get_transforms_async(self.h, C.c_void_p(host_ptr)), "gb_get_transforms_async")

    def get_transforms(self) -> np.ndarray:
        out = np.zeros((self.total_bodies, 4), dtype=np.float32)
        self.get_transforms_ptr(out.ctypes.data)
        return out


def sincos(x: np.ndarray):
    """The project sin/cos evaluated on the GPU."""
    lib = _lib.load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    s, c = np.zeros_like(x), np.zeros_like(x)
    _lib.check(lib.gb_sincos(x, s, c, len(x)), "gb_sincos")
    return s, c


def collide(type_a, shape_a, n_a, xf_a, type_b, shape_b, n_b, xf_b):
    """Narrowphase on the GPU for arrays of shape pairs (see gb_collide)."""
    lib = _lib.load()
    n = len(type_a)
    f = lambda a, shp, dt: np.ascontiguousarray(np.asarray(a, dtype=dt).reshape(shp))
    oi = np.zeros((n, 4), dtype=np.int32)
    of = np.zeros((n, 12), dtype=np.float32)
    _lib.check(lib.gb_collide(n, f(type_a, n, np.int32), f(shape_a, (n, 16), np.float32), f(n_a, n, np.int32),
                              f(xf_a, (n, 4), np.float32), f(type_b, n, np.int32), f(shape_b, (n, 16), np.float32),
                              f(n_b, n, np.int32), f(xf_b, (n, 4), np.float32), oi, of), "gb_collide")
    return oi, of


def collide_noalloc(type_a, shape_a, n_a, xf_a, type_b, shape_b, n_b, xf_b):
    """``collide`` through gb_collide_noalloc: the same narrowphase with inputs and outputs staged in
    the library's fixed device buffer (at most ``_lib.COLLIDE_NOALLOC_MAX_PAIRS`` pairs per call)."""
    lib = _lib.load()
    n = len(type_a)
    f = lambda a, shp, dt: np.ascontiguousarray(np.asarray(a, dtype=dt).reshape(shp))
    oi = np.zeros((n, 4), dtype=np.int32)
    of = np.zeros((n, 12), dtype=np.float32)
    _lib.check(lib.gb_collide_noalloc(n, f(type_a, n, np.int32), f(shape_a, (n, 16), np.float32),
                                      f(n_a, n, np.int32), f(xf_a, (n, 4), np.float32), f(type_b, n, np.int32),
                                      f(shape_b, (n, 16), np.float32), f(n_b, n, np.int32),
                                      f(xf_b, (n, 4), np.float32), oi, of), "gb_collide_noalloc")
    return oi, of
