"""Oracle (test infrastructure only; never imported by the product).

Two CPU implementations of the Box2D 2.3.2 step, driven through the same C-ABI shape:

* ``ReferenceWorld`` - the UNMODIFIED reference (box2dref from the reference tree) compiled here by
  ``oracle/Makefile`` into ``oracle/_ref/``; available only where the reference tree exists (it is
  the source of the committed golden vectors under ``tests/golden/``). ``trig="libm"`` links glibc's
  sinf/cosf, ``trig="project"`` links the project trig (``oracle/trig.c``) in their place.
* ``PortWorld`` - the project's own CPU restatement (``oracle/port/``), built on any machine into
  ``oracle/_build/liboracle.so``; ``trig`` selects the same two sin/cos choices.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_tree() -> str:
    """The reference's Regression/box2d-ref directory as oracle/reference_tree.sh locates it (the
    B2_REFERENCE_TREE environment variable, else the recipe's own fallback), or "" when absent."""
    try:
        out = subprocess.run(["sh", os.path.join(HERE, "reference_tree.sh")], capture_output=True, text=True,
                             env=os.environ.copy(), timeout=30)
    except (OSError, subprocess.SubprocessError):
        return ""
    return out.stdout.strip() if out.returncode == 0 else ""


REF_TREE = _reference_tree()

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port(quiet: bool = True) -> str:
    """Compile the CPU restatement (runs make; cheap when up to date)."""
    out = subprocess.run(["make", "-C", HERE, "port"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "_build", "liboracle.so")


def reference_available() -> bool:
    return bool(REF_TREE) and os.path.isdir(os.path.join(REF_TREE, "Box2DRef"))


def build_reference() -> None:
    """Compile the reference from its own sources (only where the reference tree exists)."""
    if not reference_available():
        raise RuntimeError("reference tree not present")
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={REF_TREE}", "-j8"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)


_LIBS: dict = {}


# entry points only the reference driver has (queries of the reference's own classes)
REFERENCE_ONLY = {"fixture_query"}


def _declare(lib, p: str) -> None:
    vp = C.c_void_p
    sig = {
        "create": (vp, [C.c_float, C.c_float]),
        "destroy": (None, [vp]),
        "config": (None, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "build": (None, [vp, C.c_int, _i32p, _f32p, _i32p, C.c_int, _i32p, _i32p, _f32p, _i32p, _f32p, _i32p,
                         C.c_int, _i32p, _i32p, _f32p, _i32p]),
        "step": (None, [vp, C.c_float, C.c_int, C.c_int]),
        "body_count": (C.c_int, [vp]),
        "contact_count": (C.c_int, [vp]),
        "get_bodies": (None, [vp, _f32p]),
        "get_contacts": (C.c_int, [vp, _i32p, _f32p, C.c_int]),
        "get_proxies": (None, [vp, _i32p, _f32p]),
        "collide": (C.c_int, [C.c_int, _f32p, C.c_int, _f32p, C.c_int, _f32p, C.c_int, _f32p, _i32p, _f32p]),
        "polygon": (None, [C.c_int, _f32p, C.c_int, C.c_float, _f32p]),
        "toi": (None, [C.c_int, _f32p, C.c_int, _f32p, C.c_int, _f32p, C.c_int, _f32p, C.c_float, _f32p]),
        "sincosf": (None, [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "step_many": (None, [C.POINTER(vp), C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]),
        "body_edit": (None, [vp, C.c_int, C.c_int, C.c_int, _f32p]),
    }
    sig["joint"] = (C.c_int, [vp, C.c_int, C.c_int, C.c_int, _f32p, C.c_int])
    sig["body"] = (C.c_int, [vp, C.c_int, _f32p, C.c_int])
    sig["fixture"] = (C.c_int, [vp, C.c_int, C.c_int, _f32p, C.c_int, _f32p, _i32p])
    sig["set_presolve_rule"] = (None, [vp, _i32p, C.c_int])
    sig["set_filter_rule"] = (None, [vp, C.c_int, C.c_int])
    sig["set_settings"] = (None, [vp, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int])
    sig["clear_forces"] = (None, [vp])
    sig["body_set"] = (None, [vp, C.c_int, C.c_int, _f32p])
    sig["tree_stats"] = (None, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)])
    sig["body_info"] = (None, [vp, C.c_int, _f32p, C.POINTER(C.c_int)])
    sig["fixture_set"] = (None, [vp, C.c_int, C.c_int, _f32p])
    sig["shift_origin"] = (None, [vp, C.c_float, C.c_float])
    sig["joint_set"] = (C.c_int, [vp, C.c_int, C.c_int, _f32p])
    sig["joint_reaction"] = (None, [vp, C.c_int, C.c_float, _f32p])
    sig["fixture_query"] = (None, [vp, C.c_int, C.c_int, _f32p, _f32p])
    for kind in ("body", "joint", "fixture"):
        sig["destroy_" + kind] = (C.c_int, [vp, C.c_int, _i32p, C.c_int])
    if p == "rw_":
        sig["query_aabb"] = (C.c_int, [vp, _f32p, _i32p, C.c_int])
        sig["raycast"] = (C.c_int, [vp, _f32p, _f32p])
    if p == "po_":
        sig["set_trig"] = (None, [C.c_int])
        sig["record_events"] = (None, [vp, C.c_int])
        sig["get_pairs"] = (C.c_int, [vp, _i32p, C.c_int])
        sig["get_events"] = (C.c_int, [vp, _i32p, _f32p, C.c_int])
    for name, (res, args) in sig.items():
        if name in REFERENCE_ONLY and not hasattr(lib, p + name):
            continue
        fn = getattr(lib, p + name)
        fn.restype = res
        fn.argtypes = args


def load(kind: str = "port", trig: str = "project"):
    """Return (ctypes library, symbol prefix) for kind 'port' or 'reference'."""
    key = (kind, trig)
    if key in _LIBS:
        return _LIBS[key]
    if kind == "port":
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            build_port()
        # one private copy per trig mode: the mode is a process-wide switch inside the library
        lib = C.CDLL(path, mode=C.RTLD_LOCAL) if trig == "project" else C.CDLL(_copy_for(path, trig), mode=C.RTLD_LOCAL)
        _declare(lib, "po_")
        lib.po_set_trig(1 if trig == "project" else 0)
        res = (lib, "po_")
    elif kind == "reference":
        name = "libref_proj.so" if trig == "project" else "libref_libm.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            build_reference()
        lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        _declare(lib, "rw_")
        res = (lib, "rw_")
    else:
        raise ValueError(kind)
    _LIBS[key] = res
    return res


def _copy_for(path: str, tag: str) -> str:
    dst = path.replace(".so", f"_{tag}.so")
    if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(path):
        import shutil
        shutil.copyfile(path, dst)
    return dst


class OracleWorld:
    """One world of either CPU implementation, built from a ``box2dpp_gb300.scenes.Scene``."""

    def __init__(self, scene, kind: str = "port", trig: str = "project"):
        self.lib, self.p = load(kind, trig)
        self.kind = kind
        f = self._fn
        self.h = f("create")(float(scene.gravity[0]), float(scene.gravity[1]))
        f("config")(self.h, int(scene.allow_sleep), int(scene.warm_starting), int(scene.continuous),
                    int(scene.sub_stepping))
        a = scene.arrays()
        typed = bool(len(a["joint_type"])) and bool((a["joint_type"] != 0).any())
        nj = 0 if typed else len(a["joint_a"])
        f("build")(self.h, len(a["body_type"]), a["body_type"], a["body_f"], a["body_flags"],
                   len(a["fix_body"]), a["fix_body"], a["fix_type"], a["fix_shape"], a["fix_n"], a["fix_mat"],
                   a["fix_filt"], nj, a["joint_a"], a["joint_b"], a["joint_f"], a["joint_flags"])
        if typed:
            for j in range(len(a["joint_a"])):
                f("joint")(self.h, int(a["joint_type"][j]), int(a["joint_a"][j]), int(a["joint_b"][j]),
                           np.ascontiguousarray(a["joint_f"][j]), int(a["joint_flags"][j]))
        self.n_fixtures = len(a["fix_body"])

    def _fn(self, name):
        return getattr(self.lib, self.p + name)

    def __del__(self):
        try:
            self._fn("destroy")(self.h)
        except Exception:
            pass

    def step(self, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> None:
        self._fn("step")(self.h, dt, vi, pi)

    def add_body(self, type_: int, f, flags: int) -> int:
        """b2World::CreateBody between steps: f = the 9 floats of the body encoding, returns its index."""
        return self._fn("body")(self.h, int(type_), np.ascontiguousarray(f, dtype=np.float32), int(flags))

    def add_fixture(self, body: int, type_: int, shape, n: int, mat, filt) -> int:
        """b2Body::CreateFixture between steps (one fixture record; no chains), returns its index."""
        s = np.zeros(16, dtype=np.float32)
        s[:len(shape)] = shape
        self.n_fixtures += 1
        return self._fn("fixture")(self.h, int(body), int(type_), s, int(n), np.asarray(mat, dtype=np.float32),
                                   np.asarray(filt, dtype=np.int32))

    def set_filter_rule(self, modulus: int, first_other: int) -> None:
        """A b2ContactFilter: fixtures below first_other keep the default filter; any other pair
        collides unless (fixtureA + fixtureB) % modulus == 0."""
        self._fn("set_filter_rule")(self.h, int(modulus), int(first_other))

    def set_settings(self, gravity, allow_sleep: bool, warm_starting: bool, continuous: bool, sub_stepping: bool,
                     auto_clear_forces: bool) -> None:
        """b2World::SetGravity, SetAllowSleeping, SetWarmStarting, SetContinuousPhysics, SetSubStepping
        and SetAutoClearForces between steps."""
        self._fn("set_settings")(self.h, float(gravity[0]), float(gravity[1]), int(allow_sleep), int(warm_starting),
                                 int(continuous), int(sub_stepping), int(auto_clear_forces))

    def fixture_query(self, fixture: int, op: int, inp=()) -> np.ndarray:
        """b2Fixture::TestPoint (op 0), RayCast (op 1: p1, p2, maxFraction -> hit, normal, fraction) or
        GetAABB (op 2) of a fixture's first child; the reference driver only."""
        v = np.zeros(8, dtype=np.float32)
        v[:len(inp)] = inp
        out = np.zeros(4, dtype=np.float32)
        self._fn("fixture_query")(self.h, int(fixture), int(op), v, out)
        return out

    def joint_reaction(self, joint: int, inv_dt: float) -> np.ndarray:
        """b2Joint::GetReactionForce and GetReactionTorque: (force x, force y, torque) as float32."""
        out = np.zeros(3, dtype=np.float32)
        self._fn("joint_reaction")(self.h, int(joint), float(inv_dt), out)
        return out

    def joint_set(self, joint: int, prop: int, value=0.0) -> None:
        """A joint setter between steps (prop: the C-ABI's GB_JOINT_*; value a number or a pair)."""
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        if self._fn("joint_set")(self.h, int(joint), int(prop), v) != 0:
            raise ValueError(f"joint {joint} has no property {prop}")

    def shift_origin(self, x: float, y: float) -> None:
        """b2World::ShiftOrigin(b2Vec2(x, y))."""
        self._fn("shift_origin")(self.h, float(x), float(y))

    def fixture_set(self, fixture: int, prop: int, value=0.0):
        """A b2Fixture change between steps (prop: 0 SetFriction, 1 SetRestitution, 2 SetDensity,
        3 SetSensor, 4 SetFilterData with value = (category, mask, group))."""
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        self._fn("fixture_set")(self.h, int(fixture), int(prop), v)
        return np.zeros((0, 3), dtype=np.int32)

    def body_info(self, body: int):
        """(mass, inertia, local center x, y, linear damping, angular damping, gravity scale) and the
        flags (type | 4 bullet | 8 fixed rotation | 16 sleeping allowed | 32 active) of a body."""
        out = np.zeros(7, dtype=np.float32)
        fl = C.c_int()
        self._fn("body_info")(self.h, int(body), out, C.byref(fl))
        return out, fl.value

    def tree_stats(self):
        """b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality: (height, balance, quality)."""
        h, b, q = C.c_int(), C.c_int(), C.c_float()
        self._fn("tree_stats")(self.h, C.byref(h), C.byref(b), C.byref(q))
        return h.value, b.value, np.float32(q.value)

    def clear_forces(self) -> None:
        """b2World::ClearForces."""
        self._fn("clear_forces")(self.h)

    def body_set(self, body: int, prop: int, value=0.0):
        """A b2Body property change between steps (prop: the C-ABI's GB_BODY_* code: 0 SetType,
        1 SetActive, 2 SetFixedRotation, 3 SetBullet, 4 SetSleepingAllowed, 5 SetLinearDamping,
        6 SetAngularDamping, 7 SetGravityScale, 8 SetMassData with value = (mass, center x, center y,
        inertia), 9 ResetMassData). Returns no listener calls (the reference driver's EndContact calls
        go to its recorded events, when recording)."""
        v = np.zeros(4, dtype=np.float32)
        vals = np.atleast_1d(np.asarray(value, dtype=np.float32))
        v[:len(vals)] = vals
        self._fn("body_set")(self.h, int(body), int(prop), v)
        return np.zeros((0, 3), dtype=np.int32)

    def set_presolve_rule(self, bits) -> None:
        """A PreSolve listener applying a rule per fixture pair (bits per fixture: 1 ghost, 2 ice,
        4 bouncy; a contact between two fixtures sharing a bit is disabled, gets friction 0 or
        restitution 0.9)."""
        b = np.ascontiguousarray(bits, dtype=np.int32)
        self._fn("set_presolve_rule")(self.h, b, len(b))

    def _destroy(self, kind: str, index: int):
        calls = np.zeros((64, 2), dtype=np.int32)
        n = self._fn("destroy_" + kind)(self.h, int(index), calls, 64)
        return calls[:min(n, 64)]

    def destroy_body(self, body: int) -> np.ndarray:
        """b2World::DestroyBody; returns the destruction listener's calls {0 joint / 1 fixture, index}."""
        return self._destroy("body", body)

    def destroy_joint(self, joint: int) -> np.ndarray:
        """b2World::DestroyJoint (no listener calls)."""
        return self._destroy("joint", joint)

    def destroy_fixture(self, fixture: int) -> np.ndarray:
        """b2Body::DestroyFixture (no listener calls)."""
        return self._destroy("fixture", fixture)

    def body_edit(self, op: int, body: int, values, wake: bool = True) -> None:
        """A b2Body state change between steps (op: the C-ABI's GB_EDIT_* code)."""
        v = np.zeros(4, dtype=np.float32)
        v[:len(values)] = values
        self._fn("body_edit")(self.h, int(op), int(body), int(bool(wake)), v)

    def bodies(self) -> np.ndarray:
        n = self._fn("body_count")(self.h)
        out = np.zeros((n, 12), dtype=np.float32)
        self._fn("get_bodies")(self.h, out)
        return out

    def contacts(self):
        n = self._fn("contact_count")(self.h)
        ints = np.zeros((max(n, 1), 8), dtype=np.int32)
        flts = np.zeros((max(n, 1), 12), dtype=np.float32)
        got = self._fn("get_contacts")(self.h, ints, flts, n)
        return ints[:got], flts[:got]

    def proxies(self):
        ids = np.zeros(max(self.n_fixtures, 1), dtype=np.int32)
        fat = np.zeros((max(self.n_fixtures, 1), 4), dtype=np.float32)
        self._fn("get_proxies")(self.h, ids, fat)
        return ids[:self.n_fixtures], fat[:self.n_fixtures]

    def pairs(self) -> np.ndarray:
        n = self._fn("get_pairs")(self.h, np.zeros(2, dtype=np.int32), 0)
        out = np.zeros((max(n, 1), 2), dtype=np.int32)
        self._fn("get_pairs")(self.h, out, n)
        return out[:n]

    def query_aabb(self, box):
        """Fixture indices the reference reports for the box (lower.x, lower.y, upper.x, upper.y), sorted
        (reference build only)."""
        box = np.ascontiguousarray(box, dtype=np.float32)
        fn = self._fn("query_aabb")
        n = fn(self.h, box, np.zeros(1, np.int32), 0)
        out = np.zeros(max(n, 1), dtype=np.int32)
        fn(self.h, box, out, n)
        return out[:n]

    def raycast(self, ray):
        """(fixture or -1, [fraction, point.x, point.y, normal.x, normal.y]) of the closest hit
        (reference build only)."""
        hit = np.zeros(5, dtype=np.float32)
        f = self._fn("raycast")(self.h, np.ascontiguousarray(ray, dtype=np.float32), hit)
        return f, hit

    def record_events(self, on: bool = True) -> None:
        self._fn("record_events")(self.h, int(on))

    def events(self):
        n = self._fn("get_events")(self.h, np.zeros(3, dtype=np.int32), np.zeros(4, dtype=np.float32), 0)
        ints = np.zeros((max(n, 1), 3), dtype=np.int32)
        flts = np.zeros((max(n, 1), 4), dtype=np.float32)
        self._fn("get_events")(self.h, ints, flts, n)
        return ints[:n], flts[:n]


def step_many(worlds: list, steps: int, threads: int, dt: float = 1.0 / 60.0, vi: int = 8, pi: int = 3) -> None:
    """Step independent worlds of one kind on `threads` host threads (round-robin split)."""
    if not worlds:
        return
    lib, p = worlds[0].lib, worlds[0].p
    arr = (C.c_void_p * len(worlds))(*[w.h for w in worlds])
    getattr(lib, p + "step_many")(arr, len(worlds), dt, vi, pi, steps, threads)


def collide(kind: str, trig: str, typeA, shapeA, nA, xfA, typeB, shapeB, nB, xfB):
    lib, p = load(kind, trig)
    oi = np.zeros(4, dtype=np.int32)
    of = np.zeros(12, dtype=np.float32)
    sa = np.zeros(16, dtype=np.float32); sa[:len(shapeA)] = shapeA
    sb = np.zeros(16, dtype=np.float32); sb[:len(shapeB)] = shapeB
    r = getattr(lib, p + "collide")(typeA, sa, nA, np.asarray(xfA, dtype=np.float32), typeB, sb, nB,
                                    np.asarray(xfB, dtype=np.float32), oi, of)
    if r != 0:
        raise ValueError("unsupported shape pair")
    return oi, of


def polygon(kind: str, type_, shape, n, density=1.0):
    lib, p = load(kind, "project")
    s = np.zeros(16, dtype=np.float32); s[:len(shape)] = shape
    out = np.zeros(40, dtype=np.float32)
    getattr(lib, p + "polygon")(type_, s, n, density, out)
    return out


def toi(kind: str, trig: str, typeA, shapeA, nA, sweepA, typeB, shapeB, nB, sweepB, tmax=1.0):
    lib, p = load(kind, trig)
    sa = np.zeros(16, dtype=np.float32); sa[:len(shapeA)] = shapeA
    sb = np.zeros(16, dtype=np.float32); sb[:len(shapeB)] = shapeB
    out = np.zeros(2, dtype=np.float32)
    getattr(lib, p + "toi")(typeA, sa, nA, np.asarray(sweepA, dtype=np.float32), typeB, sb, nB,
                            np.asarray(sweepB, dtype=np.float32), tmax, out)
    return int(out[0]), float(out[1])


def sincosf(kind: str, trig: str, x: float):
    lib, p = load(kind, trig)
    s, c = C.c_float(), C.c_float()
    getattr(lib, p + "sincosf")(x, C.byref(s), C.byref(c))
    return s.value, c.value
