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


def tree_cases():
    """(name, scene factory, steps, ops by step) of the tree_stats.npz golden cases."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.tree_cases()


def tree_stats_mismatch(world, steps: int, script: dict, g, name: str):
    """Steps `world` (oracle or device) with the case's ops and compares its tree height, balance and
    quality (bits) with the golden ones after every step; returns the first differing step or None."""
    hb, q = g[f"{name}_hb"], g[f"{name}_quality"]
    for s in range(1, steps + 1):
        if s in script:
            apply_ops(world, script[s])
        world.step(DT, VI, PI)
        h, b, qq = world.tree_stats()
        if (h, b) != tuple(int(x) for x in hb[s - 1]) or np.float32(qq).view(np.uint32) != q[s - 1].view(np.uint32):
            return s, (h, b, qq), (hb[s - 1], q[s - 1])
    return None


def first_divergence(world, steps: int, golden_digests: np.ndarray):
    """Step index (1-based) where `world`'s state digest first differs from the golden one, or None."""
    for s in range(1, steps + 1):
        world.step(DT, VI, PI)
        b = world.bodies()
        ci, cf = world.contacts()
        if not np.array_equal(digest(b, ci, cf), golden_digests[s - 1]):
            return s
    return None


# op codes of gb_body_edit (GB_EDIT_*)
SET_TRANSFORM, SET_LINEAR_VELOCITY, SET_ANGULAR_VELOCITY, SET_AWAKE = 0, 1, 2, 3
APPLY_FORCE, APPLY_FORCE_TO_CENTER, APPLY_TORQUE, APPLY_LINEAR_IMPULSE, APPLY_ANGULAR_IMPULSE = 4, 5, 6, 7, 8
MOUSE_TARGET = 9  # the body field is the mouse joint's index


def mouse_script():
    """{step: [(op, body, values, wake)]} for the pulley_mouse scene (mouse joints 2 and 3): the stiff
    joint's target dragged along a circle every 3 steps, the weak one lifted and dropped, an impulse
    in between, and a target set on a body put to sleep (SetTarget wakes it)."""
    import math

    script = {}
    for s in range(20, 200, 3):
        t = (s - 20) * 0.05
        tx = float(np.float32(16.25 + 2.0 * math.sin(t)))
        ty = float(np.float32(6.25 + 1.5 - 1.5 * math.cos(t)))
        script.setdefault(s, []).append((MOUSE_TARGET, 2, (tx, ty), True))
    script.setdefault(50, []).append((MOUSE_TARGET, 3, (21.0, 4.0), True))
    script.setdefault(120, []).append((MOUSE_TARGET, 3, (19.0, 0.5), True))
    script.setdefault(130, []).append((APPLY_LINEAR_IMPULSE, 7, (0.0, 3.0, 20.0, 0.6), True))
    script.setdefault(320, []).append((SET_AWAKE, 7, (0.0,), True))
    script.setdefault(330, []).append((MOUSE_TARGET, 2, (14.0, 3.0), True))
    script.setdefault(331, []).append((MOUSE_TARGET, 3, (20.0, 6.0), True))
    return script


def edit_scene():
    """A 10-row pyramid on an edge ground with a kinematic paddle, sleep on: the b2Body edit cases."""
    from box2dpp_gb300 import scenes

    s = scenes.pyramid(10)
    k = s.body(scenes.KINEMATIC, -15.0, 3.0, vx=1.0)
    s.fixture(k, scenes.BOX, [2.0, 0.25], 2)
    return s


def edit_script():
    """{step: [(op, body, values, wake)]} applied before that step: every edit kind, on dynamic,
    static (body 0) and kinematic (the last body) targets, on awake and sleeping bodies."""
    kin = 56  # 1 ground + 55 boxes, then the paddle
    return {
        5: [(APPLY_LINEAR_IMPULSE, 3, (2.0, 9.0, 0.3, 0.9), True), (APPLY_ANGULAR_IMPULSE, 8, (1.5,), True),
            (SET_LINEAR_VELOCITY, 0, (3.0, 0.0), True)],
        20: [(SET_TRANSFORM, 55, (6.0, 14.0, 0.7), True), (SET_ANGULAR_VELOCITY, 55, (2.0,), True),
             (APPLY_FORCE, 12, (300.0, 40.0, 0.2, 1.0), True), (APPLY_TORQUE, 13, (25.0,), False),
             (APPLY_FORCE_TO_CENTER, 14, (-200.0, 0.0), True)],
        40: [(SET_LINEAR_VELOCITY, kin, (-2.0, 0.5), True), (SET_ANGULAR_VELOCITY, kin, (0.3,), True),
             (SET_AWAKE, 20, (0.0,), True), (SET_TRANSFORM, 30, (-8.0, 0.6, 0.0), True)],
        60: [(APPLY_LINEAR_IMPULSE, 20, (0.0, 5.0, 0.0, 0.0), False), (APPLY_FORCE, 21, (0.0, 500.0, 0.0, 0.0), True)],
        300: [(APPLY_LINEAR_IMPULSE, 25, (4.0, 4.0, 0.0, 0.0), False), (APPLY_TORQUE, 26, (10.0,), False),
              (SET_AWAKE, 27, (1.0,), True), (APPLY_ANGULAR_IMPULSE, 28, (3.0,), True)],
        310: [(SET_TRANSFORM, kin, (15.0, 3.0, 0.2), True), (SET_LINEAR_VELOCITY, 40, (0.0, 0.0), True)],
    }


def destroy_script():
    """{step: [op]} applied before that step to scenes.destroy_mix: every kind of destruction, and new
    bodies created after destructions (their proxies take the freed tree nodes). Ops: ("body", i),
    ("joint", i), ("fixture", i) destroy; ("add", type, f9, fixtures) creates a body whose fixtures
    are (type, shape, n, density) records."""
    box = (3, [0.4, 0.4], 2, 1.0)
    circle = (0, [0.0, 0.0, 0.3], 0, 1.0)
    tri = (2, [-0.4, -0.3, 0.4, -0.3, 0.0, 0.45], 3, 2.0)

    def add(x, y, *fixtures):
        return ("add", 2, [x, y, 0.1, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0], list(fixtures))

    return {
        30: [("body", 12)],                      # a pyramid box in the second row, touching four
        45: [("joint", 3)],                      # the chain splits
        60: [("fixture", 48)],                   # the two-fixture body loses its circle
        75: [add(-2.0, 14.0, box), add(0.0, 15.0, circle), add(2.0, 14.0, tri)],
        90: [("body", 43)],                      # a link with two joints: goodbyes, then its fixture
        100: [("joint", 8)],                     # the tied pair may now collide
        110: [("body", 37)],                     # the static ledge
        130: [("body", 5), ("body", 20), ("body", 51), add(-4.0, 12.0, box, circle), add(4.0, 12.0, tri),
              add(0.0, 18.0, circle), add(1.0, 20.0, box)],
        150: [("body", 60), ("fixture", 64)],
    }


def settings_script():
    """{step: [op]} applied before that step to scenes.destroy_mix: the b2World settings changed
    between steps. Ops: ("settings", gx, gy, allow_sleep, warm_starting, continuous, sub_stepping,
    auto_clear_forces), ("force", body, fx, fy, torque) (b2Body::ApplyForceToCenter + ApplyTorque,
    waking the body), ("clear_forces",) (b2World::ClearForces)."""
    def st(gx, gy, sleep=1, warm=1, cont=1, sub=0, clear=1):
        return ("settings", gx, gy, sleep, warm, cont, sub, clear)

    return {
        40: [st(3.0, -6.0)],                                    # gravity changes
        60: [st(0.0, -10.0)],
        100: [st(0.0, -10.0, clear=0), ("force", 50, 0.0, 12.0, 1.0)],   # forces kept between steps
        120: [("clear_forces",), st(0.0, -10.0, warm=0)],       # cleared; no warm start
        140: [st(0.0, -10.0, cont=0)],                          # no continuous collision
        160: [st(0.0, -10.0, sub=1)],                           # single-event sub-stepping
        180: [st(0.0, -10.0)],                                  # all back on
        300: [st(0.0, -10.0, sleep=0)],                         # sleep off: the sleeping bodies wake
        320: [st(-2.0, -9.0)],                                  # sleep on again, another gravity
    }


def body_props_script():
    """{step: [op]} applied before that step to scenes.destroy_mix: b2Body properties changed between
    steps. Op ("prop", body, prop, value): prop 0 SetType (0 static, 1 kinematic, 2 dynamic),
    1 SetActive, 2 SetFixedRotation, 3 SetBullet, 4 SetSleepingAllowed, 5 SetLinearDamping,
    6 SetAngularDamping, 7 SetGravityScale, 8 SetMassData (value: mass, center x, center y, inertia
    about the body origin), 9 ResetMassData."""
    return {
        30: [("prop", 12, 0, 0.0)],                              # a pyramid box turns static
        45: [("prop", 43, 1, 0.0)],                              # a chain link leaves the world
        60: [("prop", 47, 2, 1.0), ("prop", 50, 7, -0.5)],       # fixed rotation; a circle rises
        75: [("prop", 43, 1, 1.0)],                              # the link comes back
        90: [("prop", 12, 0, 2.0)],                              # the box is dynamic again
        100: [("prop", 37, 0, 2.0)],                             # the static ledge falls
        110: [("prop", 48, 0, 1.0)],                             # a tied circle turns kinematic
        120: [("prop", 51, 3, 1.0), ("prop", 52, 5, 3.0), ("prop", 53, 6, 2.0)],
        130: [("prop", 47, 8, (3.0, 0.2, -0.1, 2.5))],            # user mass data, shifted center
        140: [("prop", 47, 2, 0.0), ("prop", 50, 7, 1.0)],
        160: [("prop", 30, 1, 0.0)],                             # a loaded pyramid box leaves
        170: [("prop", 47, 9, 0.0), ("prop", 13, 8, (0.5, 0.0, 0.0, 0.0))],  # mass from fixtures; no inertia
        200: [("prop", 48, 0, 2.0), ("prop", 30, 1, 1.0)],
        220: [("prop", 13, 9, 0.0)],
        250: [("prop", 5, 4, 0.0)],                              # one body may not sleep
        300: [("prop", 5, 4, 1.0)],
    }


def fixture_props_script():
    """{step: [op]} applied before that step to scenes.destroy_mix: b2Fixture properties changed between
    steps. Op ("fix", fixture, prop, value): prop 0 SetFriction, 1 SetRestitution, 2 SetDensity,
    3 SetSensor, 4 SetFilterData (value: category, mask, group). Fixtures: 1..36 the pyramid's boxes,
    47 and 48 the two-fixture body's box and circle, 49 and 50 the tied pair, 51.. the drop."""
    return {
        30: [("fix", 9, 3, 1.0)],                                   # a loaded box becomes a sensor
        34: [("fix", 9, 3, 0.0)],                                   # solid again, sunk into the pile
        50: [("fix", 20, 0, 0.0), ("fix", 51, 1, 0.8)],              # no friction; a bouncy circle
        60: [("fix", 52, 4, (1.0, 0xFFFF, -5.0)), ("fix", 53, 4, (1.0, 0xFFFF, -5.0))],  # a group
        80: [("fix", 47, 2, 5.0), ("prop", 47, 9, 0.0)],             # density, then the mass reset
        90: [("fix", 30, 4, (2.0, 0xFFFE, 0.0))],                    # a box no longer meets category 1
        94: [("fix", 30, 4, (1.0, 0xFFFF, 0.0))],                    # and meets it again, overlapping
        150: [("fix", 52, 4, (1.0, 0xFFFF, 0.0))],
        200: [("fix", 48, 3, 1.0), ("fix", 49, 0, 0.9)],
    }


def shift_script():
    """{step: [op]} applied before that step to scenes.pulley_mouse: b2World::ShiftOrigin, op ("shift", x,
    y) (bodies, the mouse joint's target, the pulley's ground anchors and the broadphase move)."""
    return {40: [("shift", 10.0, -3.0)], 120: [("shift", -25.5, 7.25)], 200: [("shift", 0.1, 0.0)]}


def joint_scripts():
    """Joint setters between steps, {case: (scene factory, steps, {step: [op]})}. Op ("jset", j, prop,
    value): prop 0 motor speed, 1 maximum motor torque (force for a prismatic joint), 2 enable motor,
    3 enable limit, 4 limits (lower, upper), 5 length, 6 spring frequency, 7 damping ratio, 8 maximum
    length, 9 maximum force, 10 maximum torque, 11 linear offset (x, y), 12 angular offset,
    13 correction factor, 14 ratio."""
    from box2dpp_gb300 import scenes

    zoo = {  # joints 0, 1 wheels, 2..6 ropes, 7..9 friction, 10 motor
        40: [("jset", 0, 0, -20.0), ("jset", 0, 1, 50.0), ("jset", 1, 2, 1.0), ("jset", 1, 0, -10.0)],
        60: [("jset", 0, 6, 2.0), ("jset", 0, 7, 0.3)],
        80: [("jset", 3, 8, 0.5)],
        100: [("jset", 8, 9, 0.0), ("jset", 8, 10, 0.0)],
        120: [("jset", 10, 11, (3.0, 2.0)), ("jset", 10, 12, 0.7), ("jset", 10, 13, 0.1),
              ("jset", 10, 9, 200.0), ("jset", 10, 10, 100.0)],
        160: [("jset", 0, 2, 0.0)],
    }
    prismatic = {  # joints 0..5 and 7 prismatic, 6 revolute
        40: [("jset", 0, 0, 2.0), ("jset", 0, 1, 100.0), ("jset", 2, 2, 1.0)],
        60: [("jset", 1, 4, (-0.5, 0.5)), ("jset", 3, 3, 0.0)],
        90: [("jset", 6, 2, 1.0), ("jset", 6, 0, 3.0), ("jset", 6, 1, 200.0), ("jset", 6, 4, (-0.3, 0.3)),
             ("jset", 6, 3, 1.0)],
        120: [("jset", 1, 3, 0.0), ("jset", 6, 4, (-0.3, 0.3))],  # the same limits again: no change
    }
    mix = {  # joints 0..3 distance, 4..13 weld, 14 revolute
        40: [("jset", 0, 5, 2.5), ("jset", 0, 6, 4.0), ("jset", 0, 7, 0.5), ("jset", 4, 6, 3.0)],
        90: [("jset", 1, 5, 0.5), ("jset", 5, 7, 0.9)],
    }
    return {"joint_props_zoo": (lambda: scenes.joint_zoo(scenes.SplitMix64(6)), 220, zoo),
            "joint_props_prismatic": (lambda: scenes.prismatic_mix(scenes.SplitMix64(5)), 200, prismatic),
            "joint_props_mix": (lambda: scenes.joint_mix(scenes.SplitMix64(3)), 160, mix)}


def apply_ops(world, ops, w: int = 0):
    """Applies destroy_script(), settings_script(), body_props_script(), fixture_props_script(),
    shift_script() and joint_scripts() ops to an oracle world or a device world (same
    method names); returns the destruction listener's calls of the ops as (kind, index), in order."""
    calls = []
    for op in ops:
        if op[0] == "settings":
            args = ((op[1], op[2]), bool(op[3]), bool(op[4]), bool(op[5]), bool(op[6]), bool(op[7]))
            world.set_settings(*args) if w == 0 else world.set_settings(*args, w=w)
        elif op[0] == "clear_forces":
            world.clear_forces() if w == 0 else world.clear_forces(w)
        elif op[0] == "jset":
            world.joint_set(op[1], op[2], op[3]) if w == 0 else world.joint_set(op[1], op[2], op[3], w)
        elif op[0] == "shift":
            world.shift_origin(op[1], op[2]) if w == 0 else world.shift_origin(op[1], op[2], w)
        elif op[0] == "fix":
            world.fixture_set(op[1], op[2], op[3]) if w == 0 else world.fixture_set(op[1], op[2], op[3], w)
        elif op[0] == "prop":
            # a device world also returns the EndContact calls, which the oracles record with their
            # other events
            world.body_set(op[1], op[2], op[3]) if w == 0 else world.body_set(op[1], op[2], op[3], w)
        elif op[0] == "force":
            _, b, fx, fy, t = op
            if hasattr(world, "body_edits"):
                world.body_edits([(w, b, "apply_force_to_center", [fx, fy], True), (w, b, "apply_torque", [t], True)])
            else:
                world.body_edit(5, b, [fx, fy], True)
                world.body_edit(6, b, [t], True)
        elif op[0] == "add":
            b = world.add_body(op[1], op[2], 1 | 2 | 16) if w == 0 else world.add_body(op[1], op[2], 1 | 2 | 16, w)
            for (t, shape, n, density) in op[3]:
                args = (b, t, shape, n, [density, 0.4, 0.0], [1, 0xFFFF, 0, 0])
                world.add_fixture(*args) if w == 0 else world.add_fixture(*args, w)
        else:
            fn = getattr(world, "destroy_" + op[0])
            got = fn(op[1]) if w == 0 else fn(op[1], w)
            # the destruction listener's calls {kind 0 joint / 1 fixture, index}; a device world also
            # reports EndContact calls (kind 2), which the oracles record with their other events
            calls.extend([(int(c[0]), int(c[1])) for c in got if int(c[0]) in (0, 1)])
    return calls


def presolve_case():
    """The scene and the PreSolve rule bits of the split-step case: 200 circles and polygons dropped
    into an edge box (sleep on); dynamic fixture i is a ghost when i % 3 == 0, ice when i % 4 == 0 and
    bouncy when i % 5 == 0 (contacts between two ghosts are disabled, between two ice fixtures get
    friction 0, between two bouncy ones restitution 0.9). The static walls take no part, so the
    continuous phase, whose contacts always involve a static body here, never meets the rule."""
    from box2dpp_gb300 import scenes

    sc = scenes.drop(200, scenes.SplitMix64(23))
    bits = np.array([0 if i < 4 else ((i % 3 == 0) * 1 | (i % 4 == 0) * 2 | (i % 5 == 0) * 4)
                     for i in range(len(sc.fixtures))], np.int32)
    return sc, bits


def presolve_edits(world, bits, w: int = 0):
    """The rule applied to the PreSolve calls recorded by the first half of a split device step: one
    gb_contact_edit per change, by list position."""
    rec, _ = world.events(w)
    ints, _ = world.contacts(w)
    pos = {(int(a), int(b)): k for k, (a, b) in enumerate(ints[:, :2])}
    edits = []
    for kind, fa, fb in rec[:, :3]:
        if kind != 2:
            continue
        both = int(bits[fa]) & int(bits[fb])
        flags = (1 if both & 1 else 0) | (2 if both & 2 else 0) | (4 if both & 4 else 0)
        if flags:
            edits.append((w, pos[(int(fa), int(fb))], flags, 0, 0.0, 0.9, 0.0))
    return edits
