"""Seeded synthetic scenes for the Box2D step (the workloads the parity tests and the benchmark run).

A scene is a flat description of the calls a user makes on a ``b2World``: bodies in creation order,
each followed by its fixtures, then joints. It is stored as numpy arrays so that any implementation
(the GPU world, the reference, the CPU oracle) can be built from it with one bulk call:

* ``body_type`` int32[N], ``body_f`` float32[N, 9] = (x, y, angle, vx, vy, w, linearDamping,
  angularDamping, gravityScale), ``body_flags`` int32[N] (1 allowSleep, 2 awake, 4 fixedRotation,
  8 bullet, 16 active).
* ``fix_body`` int32[M] (non-decreasing: fixtures follow their body), ``fix_type`` int32[M]
  (0 circle {px, py, r}; 1 edge {v1, v2, v0, v3, hasV0, hasV3}; 2 polygon from points (hull by
  ``b2PolygonShape::Set``); 3 box {hx, hy} or {hx, hy, cx, cy, angle}), ``fix_shape`` float32[M, 16],
  ``fix_n`` int32[M], ``fix_mat`` float32[M, 3] = (density, friction, restitution), ``fix_filt``
  int32[M, 4] = (categoryBits, maskBits, groupIndex, isSensor).
* ``joint_type`` int32[J] (0 revolute, 1 distance, 2 weld, 3 prismatic), ``joint_a``/``joint_b``
  int32[J], ``joint_f`` float32[J, 12] = revolute (localAnchorA, localAnchorB, referenceAngle,
  lowerAngle, upperAngle, motorSpeed, maxMotorTorque), distance (localAnchorA, localAnchorB, length,
  frequencyHz, dampingRatio), weld (localAnchorA, localAnchorB, referenceAngle, frequencyHz,
  dampingRatio), prismatic (localAnchorA, localAnchorB, localAxisA, referenceAngle,
  lowerTranslation, upperTranslation, maxMotorForce, motorSpeed), zero-padded; ``joint_flags`` int32[J] (1 limit, 2 motor, 4 collideConnected).

Random numbers come from splitmix64 on Python integers, so a seed gives the same scene on every
machine. No public benchmark scene set exists for Box2D; these follow the workload descriptions:
a 20-row box pyramid on an edge ground, a drop of mixed circles/polygons into an edge container,
vertical box stacks, and chains of revolute-jointed links.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# b2BodyType
STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
# shape encodings of the bulk build call
CIRCLE, EDGE, POLYGON, BOX = 0, 1, 2, 3
REVOLUTE, DISTANCE, WELD, PRISMATIC, WHEEL, ROPE, FRICTION, MOTOR, MOUSE, PULLEY, GEAR = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10
DEFAULT_FLAGS = 1 | 2 | 16  # allowSleep, awake, active


class SplitMix64:
    """splitmix64 generator (Steele, Lea, Flood 2014) on Python ints: portable and seedable."""

    def __init__(self, seed: int):
        self.state = seed & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))

    def randint(self, lo: int, hi: int) -> int:
        """Integer uniform in [lo, hi] inclusive."""
        return lo + (self.next_u64() % (hi - lo + 1))


def _q(x: float) -> float:
    """Quantise a generated coordinate to a 2^-20 grid so that libm differences in the double
    cos/sin used to lay out polygon vertices cannot change the float32 scene between machines."""
    return round(x * 1048576.0) / 1048576.0


@dataclass
class Scene:
    gravity: tuple = (0.0, -10.0)
    allow_sleep: bool = True
    warm_starting: bool = True
    continuous: bool = True
    sub_stepping: bool = False
    name: str = ""
    bodies: list = field(default_factory=list)   # (type, f9, flags)
    fixtures: list = field(default_factory=list)  # (body, type, shape list, n, mat3, filt4)
    joints: list = field(default_factory=list)    # (a, b, f9, flags)

    # ------------------------------------------------------------------ building
    def body(self, type_, x, y, angle=0.0, vx=0.0, vy=0.0, w=0.0, lin_damp=0.0, ang_damp=0.0,
             gravity_scale=1.0, flags=DEFAULT_FLAGS) -> int:
        self.bodies.append((type_, [x, y, angle, vx, vy, w, lin_damp, ang_damp, gravity_scale], flags))
        return len(self.bodies) - 1

    def fixture(self, body, type_, shape, n=0, density=0.0, friction=0.2, restitution=0.0,
                category=1, mask=0xFFFF, group=0, sensor=False) -> int:
        assert body == len(self.bodies) - 1, "fixtures must follow their body"
        self.fixtures.append((body, type_, list(shape), n, [density, friction, restitution],
                              [category, mask, group, int(sensor)]))
        return len(self.fixtures) - 1

    def chain(self, body, vertices, loop=False, prev=None, next_=None, density=0.0, friction=0.2, restitution=0.0,
              category=1, mask=0xFFFF, group=0, sensor=False) -> int:
        """b2ChainShape::CreateChain (or CreateLoop) + b2Body::CreateFixture: one edge fixture per child,
        as b2ChainShape::GetChildEdge (Collision/Shapes/b2ChainShape.cpp:112-142) lays them out, ghost
        vertices included, flagged as the chain's children (shape[10]: 1 the first, 2 the next ones).
        prev/next_ are the open chain's SetPrevVertex/SetNextVertex. Returns the first child's id."""
        pts = [(float(x), float(y)) for (x, y) in vertices]
        if loop:
            verts, prev_v, next_v, has_prev, has_next = pts + [pts[0]], pts[-1], pts[1], True, True
        else:
            verts = pts
            prev_v, has_prev = (prev, True) if prev is not None else ((0.0, 0.0), False)
            next_v, has_next = (next_, True) if next_ is not None else ((0.0, 0.0), False)
        m = len(verts)
        assert m >= 2
        first = len(self.fixtures)
        for i in range(m - 1):
            v0, h0 = (verts[i - 1], True) if i > 0 else (prev_v, has_prev)
            v3, h3 = (verts[i + 2], True) if i < m - 2 else (next_v, has_next)
            shape = [verts[i][0], verts[i][1], verts[i + 1][0], verts[i + 1][1], v0[0], v0[1], v3[0], v3[1],
                     float(h0), float(h3), 1.0 if i == 0 else 2.0]
            self.fixture(body, EDGE, shape, 2, density, friction, restitution, category, mask, group, sensor)
        return first

    def revolute(self, a, b, anchor_a, anchor_b, ref_angle=0.0, lower=0.0, upper=0.0, motor_speed=0.0,
                 max_motor_torque=0.0, flags=0) -> int:
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], ref_angle, lower,
                                   upper, motor_speed, max_motor_torque, 0.0, 0.0, 0.0], flags, REVOLUTE))
        return len(self.joints) - 1

    def distance(self, a, b, anchor_a, anchor_b, length, frequency_hz=0.0, damping_ratio=0.0, flags=0) -> int:
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], length, frequency_hz,
                                   damping_ratio, 0.0, 0.0, 0.0, 0.0, 0.0], flags, DISTANCE))
        return len(self.joints) - 1

    def weld(self, a, b, anchor_a, anchor_b, ref_angle=0.0, frequency_hz=0.0, damping_ratio=0.0, flags=0) -> int:
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], ref_angle, frequency_hz,
                                   damping_ratio, 0.0, 0.0, 0.0, 0.0, 0.0], flags, WELD))
        return len(self.joints) - 1

    def wheel(self, a, b, anchor_a, anchor_b, axis, max_motor_torque=0.0, motor_speed=0.0, frequency_hz=2.0,
              damping_ratio=0.7, flags=0) -> int:
        """b2WheelJointDef (axis in body A's frame, not normalised); flags 2 motor, 4 collideConnected."""
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], axis[0], axis[1],
                                   max_motor_torque, motor_speed, frequency_hz, damping_ratio, 0.0, 0.0], flags, WHEEL))
        return len(self.joints) - 1

    def rope(self, a, b, anchor_a, anchor_b, max_length, flags=0) -> int:
        """b2RopeJointDef: at most max_length between the anchors."""
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], max_length] + [0.0] * 7,
                            flags, ROPE))
        return len(self.joints) - 1

    def friction(self, a, b, anchor_a, anchor_b, max_force, max_torque, flags=0) -> int:
        """b2FrictionJointDef: relative motion resisted up to max_force and max_torque."""
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], max_force, max_torque]
                            + [0.0] * 6, flags, FRICTION))
        return len(self.joints) - 1

    def motor(self, a, b, linear_offset, angular_offset=0.0, max_force=1.0, max_torque=1.0, correction_factor=0.3,
              flags=0) -> int:
        """b2MotorJointDef: drives body B to linear_offset and angular_offset in body A's frame."""
        self.joints.append((a, b, [linear_offset[0], linear_offset[1], angular_offset, max_force, max_torque,
                                   correction_factor] + [0.0] * 6, flags, MOTOR))
        return len(self.joints) - 1

    def mouse(self, a, b, target, max_force, frequency_hz=5.0, damping_ratio=0.7, flags=0) -> int:
        """b2MouseJointDef: body B's point under `target` (world) is pulled to the target, which
        gb_body_edits' mouse-target op moves between steps; body A is normally a static body."""
        self.joints.append((a, b, [target[0], target[1], max_force, frequency_hz, damping_ratio] + [0.0] * 7,
                            flags, MOUSE))
        return len(self.joints) - 1

    def pulley(self, a, b, ground_a, ground_b, anchor_a, anchor_b, length_a, length_b, ratio=1.0, flags=4) -> int:
        """b2PulleyJointDef: length_a + ratio * length_b stays constant; anchors local to each body,
        ground anchors in world coordinates (the def's default collideConnected is true)."""
        self.joints.append((a, b, [ground_a[0], ground_a[1], ground_b[0], ground_b[1], anchor_a[0], anchor_a[1],
                                   anchor_b[0], anchor_b[1], length_a, length_b, ratio, 0.0], flags, PULLEY))
        return len(self.joints) - 1

    def gear(self, a, b, joint1, joint2, ratio=1.0, flags=0) -> int:
        """b2GearJointDef: couples revolute or prismatic joints joint1 and joint2 (indices of joints
        created before it) so that coordinate1 + ratio * coordinate2 stays constant; a and b are the
        definition's bodyA and bodyB (normally joint1's and joint2's body B)."""
        self.joints.append((a, b, [float(joint1), float(joint2), ratio] + [0.0] * 9, flags, GEAR))
        return len(self.joints) - 1

    def prismatic(self, a, b, anchor_a, anchor_b, axis, ref_angle=0.0, lower=0.0, upper=0.0, max_motor_force=0.0,
                  motor_speed=0.0, flags=0) -> int:
        """b2PrismaticJointDef: body B slides along axis (in body A's frame); flags 1 limit, 2 motor,
        4 collideConnected."""
        self.joints.append((a, b, [anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1], axis[0], axis[1], ref_angle,
                                   lower, upper, max_motor_force, motor_speed, 0.0], flags, PRISMATIC))
        return len(self.joints) - 1

    @property
    def joint_types(self) -> set:
        return {j[4] for j in self.joints}

    # ------------------------------------------------------------------ arrays
    def arrays(self) -> dict:
        nb, nf, nj = len(self.bodies), len(self.fixtures), len(self.joints)
        a = {
            "body_type": np.array([b[0] for b in self.bodies], dtype=np.int32).reshape(nb),
            "body_f": np.array([b[1] for b in self.bodies], dtype=np.float32).reshape(nb, 9),
            "body_flags": np.array([b[2] for b in self.bodies], dtype=np.int32).reshape(nb),
            "fix_body": np.array([f[0] for f in self.fixtures], dtype=np.int32).reshape(nf),
            "fix_type": np.array([f[1] for f in self.fixtures], dtype=np.int32).reshape(nf),
            "fix_shape": np.zeros((nf, 16), dtype=np.float32),
            "fix_n": np.array([f[3] for f in self.fixtures], dtype=np.int32).reshape(nf),
            "fix_mat": np.array([f[4] for f in self.fixtures], dtype=np.float32).reshape(nf, 3),
            "fix_filt": np.array([f[5] for f in self.fixtures], dtype=np.int32).reshape(nf, 4),
            "joint_type": np.array([j[4] for j in self.joints], dtype=np.int32).reshape(nj),
            "joint_a": np.array([j[0] for j in self.joints], dtype=np.int32).reshape(nj),
            "joint_b": np.array([j[1] for j in self.joints], dtype=np.int32).reshape(nj),
            "joint_f": np.array([j[2] for j in self.joints], dtype=np.float32).reshape(nj, 12),
            "joint_flags": np.array([j[3] for j in self.joints], dtype=np.int32).reshape(nj),
        }
        for i, f in enumerate(self.fixtures):
            a["fix_shape"][i, :len(f[2])] = np.array(f[2], dtype=np.float32)
        return a

    @property
    def dynamic_count(self) -> int:
        return sum(1 for b in self.bodies if b[0] == DYNAMIC)


def _settings(s: Scene, allow_sleep: bool) -> Scene:
    s.allow_sleep = allow_sleep
    return s


# ---------------------------------------------------------------------- scene kinds
def pyramid(rows: int = 20, allow_sleep: bool = True, half: float = 0.5, spacing: float = 1.125,
            density: float = 5.0, friction: float = 0.6, ground_half: float = 40.0) -> Scene:
    """A box pyramid on a static edge ground: row r (0 = bottom) has rows - r boxes of half-extent
    ``half`` spaced ``spacing`` apart, offset by half a spacing per row and 2*half higher, the bottom
    row resting on y = 0. rows = 20 gives 210 boxes."""
    s = Scene(name=f"pyramid{rows}")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-ground_half, 0.0, ground_half, 0.0, 0, 0, 0, 0, 0, 0], friction=friction)
    x0 = -(rows - 1) * spacing / 2.0
    for r in range(rows):
        for j in range(rows - r):
            x = x0 + r * spacing / 2.0 + j * spacing
            y = half + r * 2.0 * half
            b = s.body(DYNAMIC, x, y)
            s.fixture(b, BOX, [half, half], 2, density=density, friction=friction)
    return _settings(s, allow_sleep)


def stacks(n_bodies: int, rng: SplitMix64, allow_sleep: bool = True, half: float = 0.5,
           density: float = 1.0, friction: float = 0.6) -> Scene:
    """Vertical stacks of boxes of seeded height 5..40 standing 2 m apart on an edge ground."""
    h = rng.randint(5, 40)
    n_stacks = max(1, -(-n_bodies // h))
    s = Scene(name=f"stacks{n_bodies}")
    width = n_stacks * 2.0 + 10.0
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-width, 0.0, width, 0.0, 0, 0, 0, 0, 0, 0], friction=friction)
    placed = 0
    for k in range(n_stacks):
        x = (k - (n_stacks - 1) / 2.0) * 2.0
        for i in range(h):
            if placed == n_bodies:
                break
            b = s.body(DYNAMIC, x, half + i * 2.0 * half)
            s.fixture(b, BOX, [half, half], 2, density=density, friction=friction)
            placed += 1
    return _settings(s, allow_sleep)


def _random_polygon(rng: SplitMix64, radius: float) -> list:
    k = rng.randint(3, 8)
    pts = []
    for i in range(k):
        ang = 2.0 * math.pi * (i + rng.uniform(-0.3, 0.3)) / k
        pts += [_q(radius * math.cos(ang)), _q(radius * math.sin(ang))]
    return pts


def drop(n_bodies: int, rng: SplitMix64, half_size: float | None = None, allow_sleep: bool = True,
         upper_half_only: bool = False, friction: float = 0.4) -> Scene:
    """Mixed circles / convex polygons (50/50, radius U[0.25, 1]) dropped into a static square
    container of 4 edges with side 2*half_size, floor at y = 0. Polygons have 3..8 vertices on a
    jittered circle, hulled by b2PolygonShape::Set. Positions are random sequential adsorption with
    non-overlapping bounding circles (over the upper half when it can hold them, else the whole
    interior), density U[0.5, 5]."""
    if half_size is None:
        half_size = max(8.0, math.ceil(1.1 * math.sqrt(n_bodies)) + 2.0)
    L = float(half_size)
    s = Scene(name=f"drop{n_bodies}")
    g = s.body(STATIC, 0.0, 0.0)
    for v in ([-L, 0, L, 0], [-L, 0, -L, 2 * L], [L, 0, L, 2 * L], [-L, 2 * L, L, 2 * L]):
        s.fixture(g, EDGE, v + [0, 0, 0, 0, 0, 0], friction=friction)
    ylo = L if upper_half_only else 0.0
    cell = 2.1
    grid: dict = {}
    placed = []
    for i in range(n_bodies):
        is_circle = rng.uniform() < 0.5
        r = rng.uniform(0.25, 1.0)
        shape = None if is_circle else _random_polygon(rng, r)
        density = rng.uniform(0.5, 5.0)
        for _attempt in range(10000):
            x = rng.uniform(-L + 1.05, L - 1.05)
            y = rng.uniform(ylo + 1.05, 2 * L - 1.05)
            cx, cy = int(math.floor(x / cell)), int(math.floor(y / cell))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for (px, py, pr) in grid.get((cx + dx, cy + dy), ()):
                        if (px - x) ** 2 + (py - y) ** 2 < (pr + r + 0.05) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        else:
            raise RuntimeError("drop scene too dense for its container")
        x, y = _q(x), _q(y)
        grid.setdefault((cx, cy), []).append((x, y, r))
        placed.append((x, y))
        b = s.body(DYNAMIC, x, y)
        if is_circle:
            s.fixture(b, CIRCLE, [0.0, 0.0, _q(r)], density=density, friction=friction)
        else:
            s.fixture(b, POLYGON, shape, len(shape) // 2, density=density, friction=friction)
    return _settings(s, allow_sleep)


def destroy_mix(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """The scene of the destruction cases: an 8-row box pyramid and a small static ledge on an edge
    ground, a chain of 8 links hanging from a static anchor by revolute joints, a body with two
    fixtures (a box and a circle), a pair of circles tied by a distance joint that does not let them
    collide, and a loose drop of circles. Body indices: 0 ground, 1..36 the pyramid, 37 the ledge,
    38 the anchor, 39..46 the links (joints 0..7), 47 the two-fixture body, 48 and 49 the tied pair
    (joint 8), 50.. the drop."""
    s = pyramid(8, allow_sleep=allow_sleep)
    s.name = "destroy_mix"
    ledge = s.body(STATIC, 9.0, 3.0)
    s.fixture(ledge, BOX, [1.5, 0.2], 2, friction=0.5)
    anchor = s.body(STATIC, -12.0, 12.0)
    s.fixture(anchor, CIRCLE, [0.0, 0.0, 0.2])
    prev = anchor
    for k in range(8):
        b = s.body(DYNAMIC, _q(-12.0 + 0.5 + 1.0 * k), 12.0)
        s.fixture(b, BOX, [0.5, 0.1], 2, density=2.0, friction=0.3, group=-1)
        s.revolute(prev, b, [0.5 if k else 0.0, 0.0], [-0.5, 0.0])
        prev = b
    t = s.body(DYNAMIC, 9.0, 6.0, angle=0.3)
    s.fixture(t, BOX, [0.6, 0.4], 2, density=1.5, friction=0.5)
    s.fixture(t, CIRCLE, [0.5, 0.3, 0.35], density=3.0, friction=0.5)
    a = s.body(DYNAMIC, 3.0, 9.0)
    s.fixture(a, CIRCLE, [0.0, 0.0, 0.4], density=1.0, friction=0.4)
    b = s.body(DYNAMIC, 3.6, 9.5)
    s.fixture(b, CIRCLE, [0.0, 0.0, 0.4], density=1.0, friction=0.4)
    s.distance(a, b, [0.0, 0.0], [0.0, 0.0], 0.8)
    for i in range(12):
        c = s.body(DYNAMIC, _q(rng.uniform(-6.0, 6.0)), _q(10.0 + 0.9 * i))
        s.fixture(c, CIRCLE, [0.0, 0.0, _q(rng.uniform(0.2, 0.45))], density=1.0, friction=0.4)
    return s


def sensors(rng: SplitMix64, allow_sleep: bool = True, n_bodies: int = 80) -> Scene:
    """Sensor fixtures of every kind a b2Fixture can carry (isSensor, b2Fixture.h:107): a static body
    with two sensor zones across the fall (begin and end calls as bodies pass through), dynamic
    bodies of which every third carries a large proximity-sensor circle beside its solid fixture
    (sensor contacts with the ground, the zones' body and other bodies), and a kinematic sweeper
    whose only fixture is a sensor box crossing the pile. Sensor contacts are touching when the
    shapes overlap (b2TestOverlap), have no manifold, are never solved and do not wake bodies."""
    s = Scene(name="sensors")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-20.0, 0.0, 20.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.5)
    s.fixture(g, EDGE, [-20.0, 0.0, -20.0, 30.0, 0, 0, 0, 0, 0, 0], friction=0.5)
    s.fixture(g, EDGE, [20.0, 0.0, 20.0, 30.0, 0, 0, 0, 0, 0, 0], friction=0.5)
    z = s.body(STATIC, 0.0, 0.0)
    s.fixture(z, BOX, [8.0, 1.0, -6.0, 6.0, 0.0], 5, sensor=True)
    s.fixture(z, BOX, [6.0, 1.5, 7.0, 11.0, 0.3], 5, sensor=True)
    for i in range(n_bodies):
        x = _q(rng.uniform(-17.0, 17.0))
        y = _q(4.0 + 0.45 * i + rng.uniform(0.0, 0.3))
        b = s.body(DYNAMIC, x, y, angle=_q(rng.uniform(-1.0, 1.0)))
        r = _q(rng.uniform(0.25, 0.6))
        if i % 2:
            s.fixture(b, CIRCLE, [0.0, 0.0, r], density=1.0, friction=0.4)
        else:
            s.fixture(b, BOX, [r, _q(r * 0.7)], 2, density=1.0, friction=0.4)
        if i % 3 == 0:
            s.fixture(b, CIRCLE, [0.0, 0.0, _q(3.0 * r)], sensor=True)
    k = s.body(KINEMATIC, -18.0, 1.5, vx=3.0)
    s.fixture(k, BOX, [1.0, 1.5], 2, sensor=True)
    return _settings(s, allow_sleep)


def chains(n_chains: int, links: int, rng: SplitMix64, allow_sleep: bool = True, spacing: float = 3.0,
           limit: float = math.pi / 6.0) -> Scene:
    """Chains of revolute-jointed 0.1 x 0.5 m box links (limits +/-30 degrees) hanging from a static
    anchor body, with loose boxes and circles (half-extent / radius U[0.2, 0.8]) dropped beside them."""
    s = Scene(name=f"chains{n_chains}x{links}")
    g = s.body(STATIC, 0.0, 0.0)
    W = n_chains * spacing + 10.0
    s.fixture(g, EDGE, [-W, 0.0, W, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    top = links * 1.0 + 4.0
    for c in range(n_chains):
        x = (c - (n_chains - 1) / 2.0) * spacing
        prev = g
        prev_anchor = (x, top)
        for k in range(links):
            y = top - 0.5 - k * 1.0
            b = s.body(DYNAMIC, x, y)
            s.fixture(b, BOX, [0.1, 0.5], 2, density=1.0, friction=0.4, group=-(c + 1))
            anchor_world = (x, y + 0.5)
            if prev == g:
                la = anchor_world
            else:
                la = (0.0, -0.5)
            s.revolute(prev, b, la, (0.0, 0.5), 0.0, -limit, limit, flags=1)
            prev = b
    return _settings(s, allow_sleep)


def joint_mix(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Distance, weld and revolute joints together: pendulums on rigid and soft distance joints,
    rigid and soft weld chains of boxes, a revolute hinge, over a ground edge they fall onto."""
    s = Scene(name="joint_mix")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-40.0, 0.0, 40.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    anchor = s.body(STATIC, 0.0, 20.0)
    s.fixture(anchor, BOX, [0.5, 0.5], 2)
    # pendulums: rigid rods and springs of decreasing stiffness
    for k, (hz, zeta) in enumerate([(0.0, 0.0), (4.0, 0.5), (1.5, 0.1), (0.0, 0.0)]):
        x = -12.0 + 4.0 * k
        b = s.body(DYNAMIC, _q(x + rng.uniform(-1.0, 1.0)), 12.0, angle=_q(rng.uniform(-0.5, 0.5)))
        s.fixture(b, CIRCLE if k % 2 else BOX, [0.0, 0.0, 0.6] if k % 2 else [0.5, 0.4], 1 if k % 2 else 2,
                  density=1.0 + k, friction=0.4)
        length = math.hypot(x - 0.0, 8.0)
        s.distance(anchor, b, (x * 0.05, -0.5), (0.0, 0.0), _q(length), hz, zeta)
    # weld chains: rigid and soft, hanging from the anchor's neighbours, loose at the end
    for c, (hz, zeta) in enumerate([(0.0, 0.0), (6.0, 0.7)]):
        x0 = 6.0 + 6.0 * c
        top = s.body(STATIC, x0, 18.0)
        s.fixture(top, BOX, [0.2, 0.2], 2)
        prev = top
        for i in range(5):
            b = s.body(DYNAMIC, x0 + 1.0 * (i + 1), 18.0)
            s.fixture(b, BOX, [0.5, 0.12], 2, density=2.0, friction=0.3, group=-(c + 1))
            s.weld(prev, b, (0.5 if prev != top else 0.2, 0.0), (-0.5, 0.0), 0.0, hz, zeta)
            prev = b
    # a hinge with a limit, a box falling onto the arm
    arm = s.body(DYNAMIC, -20.0, 6.0)
    s.fixture(arm, BOX, [3.0, 0.2], 2, density=1.0)
    s.revolute(g, arm, (-20.0, 6.0), (0.0, 0.0), 0.0, -0.4, 0.4, flags=1)
    box = s.body(DYNAMIC, -18.0, 10.0, angle=0.3)
    s.fixture(box, BOX, [0.6, 0.6], 2, density=3.0)
    return _settings(s, allow_sleep)


def prismatic_mix(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Prismatic joints: sliders on the ground with motors against limits, a locked slider, an
    elevator lifting a platform of boxes, a slider on an unnormalised oblique axis, a piston between
    two dynamic bodies on a hinge, and boxes falling onto them."""
    s = Scene(name="prismatic_mix")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-40.0, 0.0, 40.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    # ground sliders: limits [-3, 3], motors pushing toward a limit, one without a motor, one locked
    for k, (speed, force, flags) in enumerate([(2.0, 60.0, 3), (-1.5, 30.0, 3), (0.0, 0.0, 1), (1.0, 40.0, 3)]):
        x = -24.0 + 5.0 * k
        b = s.body(DYNAMIC, x, 0.6 + 0.01 * k)
        s.fixture(b, BOX, [0.8, 0.5], 2, density=2.0, friction=0.2)
        lower, upper = (-3.0, 3.0) if k != 3 else (0.0, 0.0)
        s.prismatic(g, b, (x, 0.6), (0.0, 0.0), (1.0, 0.0), 0.0, lower, upper, force, speed, flags)
    # elevator: a platform driven up a vertical axis, boxes resting on it
    plat = s.body(DYNAMIC, 0.0, 2.0)
    s.fixture(plat, BOX, [2.5, 0.2], 2, density=3.0, friction=0.8)
    s.prismatic(g, plat, (0.0, 2.0), (0.0, 0.0), (0.0, 1.0), 0.0, -1.0, 6.0, 400.0, 1.2, 3)
    for i in range(3):
        b = s.body(DYNAMIC, _q(-1.5 + 1.5 * i + rng.uniform(-0.2, 0.2)), 2.75)
        s.fixture(b, BOX, [0.5, 0.5], 2, density=1.0, friction=0.6)
    # oblique slider: axis (2, 1) given unnormalised, no limit, gravity pulls it down the axis
    ob = s.body(DYNAMIC, 12.0, 8.0, angle=0.3)
    s.fixture(ob, BOX, [0.6, 0.3], 2, density=1.5)
    s.prismatic(g, ob, (12.0, 8.0), (0.0, 0.0), (2.0, 1.0), 0.3, 0.0, 0.0, 0.0, 0.0, 0)
    # piston: a cylinder hinged to the ground, a rod sliding in it (collide connected), a load on top
    cyl = s.body(DYNAMIC, 20.0, 3.0)
    s.fixture(cyl, BOX, [0.3, 1.5], 2, density=1.0, group=-3)
    s.revolute(g, cyl, (20.0, 1.5), (0.0, -1.5), 0.0, -0.3, 0.3, flags=1)
    rod = s.body(DYNAMIC, 20.0, 5.0)
    s.fixture(rod, BOX, [0.15, 1.2], 2, density=1.0, group=-3)
    s.prismatic(cyl, rod, (0.0, 1.0), (0.0, -1.0), (0.0, 1.0), 0.0, -0.5, 1.5, 80.0, 2.0, 3)
    load = s.body(DYNAMIC, _q(20.0 + rng.uniform(-0.3, 0.3)), 8.5)
    s.fixture(load, BOX, [0.7, 0.4], 2, density=2.0)
    # boxes falling on the sliders
    for i in range(6):
        b = s.body(DYNAMIC, _q(-25.0 + 3.5 * i + rng.uniform(-0.5, 0.5)), _q(4.0 + 1.2 * i), angle=_q(rng.uniform(-0.4, 0.4)))
        s.fixture(b, CIRCLE if i % 2 else BOX, [0.0, 0.0, 0.4] if i % 2 else [0.4, 0.4], 1 if i % 2 else 2,
                  density=1.0, friction=0.5)
    return _settings(s, allow_sleep)


def joint_zoo(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Wheel, rope, friction and motor joints: a car on sprung wheel joints (rear motor) driving over a
    bump, a rope-jointed chain swinging from an anchor, boxes held back by friction joints, a body
    pulled to an offset by a motor joint, and boxes falling among them."""
    s = Scene(name="joint_zoo")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-40.0, 0.0, 40.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.8)
    s.fixture(g, BOX, [1.0, 0.25, -8.0, 0.0, 0.3], 5, friction=0.8)
    # car: chassis and two wheels on wheel joints, axis up, springs, rear motor
    car = s.body(DYNAMIC, -20.0, 1.2)
    s.fixture(car, BOX, [1.5, 0.3], 2, density=1.0, group=-1)
    for k, (dx, flags) in enumerate([(-1.0, 2), (1.0, 0)]):
        wh = s.body(DYNAMIC, -20.0 + dx, 0.5)
        s.fixture(wh, CIRCLE, [0.0, 0.0, 0.45], 1, density=1.0, friction=0.9, group=-1)
        s.wheel(car, wh, (dx, -0.7), (0.0, 0.0), (0.0, 1.0), 40.0, -12.0, 4.0 + k, 0.7, flags)
    # rope chain: a static anchor, five boxes, rope joints of slack length
    anchor = s.body(STATIC, 5.0, 14.0)
    s.fixture(anchor, BOX, [0.3, 0.3], 2)
    prev = anchor
    for i in range(5):
        b = s.body(DYNAMIC, _q(6.2 + 1.2 * i), 14.0)
        s.fixture(b, BOX, [0.3, 0.2], 2, density=1.0, group=-2)
        s.rope(prev, b, (0.0, 0.0), (0.0, 0.0), _q(1.3 + 0.1 * rng.uniform(0.0, 1.0)))
        prev = b
    # friction joints: boxes sliding on the ground with a push (collide connected), dragged to rest
    for i, (fmax, tmax) in enumerate([(5.0, 1.0), (20.0, 4.0), (0.0, 0.0)]):
        b = s.body(DYNAMIC, 14.0 + 3.0 * i, 0.5, vx=6.0, w=3.0)
        s.fixture(b, BOX, [0.5, 0.5], 2, density=1.0, friction=0.1)
        s.friction(g, b, (14.0 + 3.0 * i, 0.5), (0.0, 0.0), fmax, tmax, flags=4)
    # motor joint: a body pulled to an offset above the ground, bounded force and torque
    m = s.body(DYNAMIC, 26.0, 1.0, angle=0.5)
    s.fixture(m, BOX, [0.8, 0.3], 2, density=2.0)
    s.motor(g, m, (28.0, 4.0), 1.0, 60.0, 10.0, 0.3)
    for i in range(5):
        b = s.body(DYNAMIC, _q(-12.0 + 5.0 * i + rng.uniform(-0.5, 0.5)), _q(6.0 + rng.uniform(0.0, 3.0)),
                   angle=_q(rng.uniform(-0.5, 0.5)))
        s.fixture(b, CIRCLE if i % 2 else BOX, [0.0, 0.0, 0.35] if i % 2 else [0.35, 0.35], 1 if i % 2 else 2,
                  density=1.0, friction=0.5)
    return _settings(s, allow_sleep)


def pulley_mouse(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Pulley and mouse joints: two pulleys (ratios 1.5 and 1) whose boxes swing, load each other and
    land, boxes falling onto the pulley boxes, and two bodies hung on mouse joints (a stiff one and one
    whose force bound the load exceeds). The mouse joints are joints 2 and 3."""
    s = Scene(name="pulley_mouse")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-30.0, 0.0, 30.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.6)
    # pulley 1: box A (2 kg) below ground anchor (-10, 20), box B (2 kg) below (-4, 20), ratio 1.5;
    # anchors at the boxes' tops, lengths 7 and 5
    a = s.body(DYNAMIC, -10.0, 12.0)
    s.fixture(a, BOX, [1.0, 1.0], 2, density=0.5)
    b = s.body(DYNAMIC, -4.0, 14.0, vx=0.5)
    s.fixture(b, BOX, [0.5, 1.0], 2, density=1.0)
    s.pulley(a, b, (-10.0, 20.0), (-4.0, 20.0), (0.0, 1.0), (0.0, 1.0), 7.0, 5.0, 1.5)
    # pulley 2: a circle and a box, ratio 1, the box off-centre so it rotates
    c = s.body(DYNAMIC, 4.0, 10.0)
    s.fixture(c, CIRCLE, [0.0, 0.0, 0.6], 1, density=1.0)
    d = s.body(DYNAMIC, 9.0, 8.0, angle=0.25)
    s.fixture(d, BOX, [0.6, 0.4], 2, density=2.0)
    s.pulley(c, d, (4.0, 18.0), (9.0, 18.0), (0.0, 0.0), (0.3, 0.4), 8.0, 10.0, 1.0)
    # mouse joints on a fixture-less static anchor (a joint to the ground body would filter the
    # ground contacts): a box held at a point of it, and a circle on a weak one that sags
    anchor = s.body(STATIC, 0.0, 0.0)
    m = s.body(DYNAMIC, 16.0, 6.0, angle=0.1)
    s.fixture(m, BOX, [0.5, 0.5], 2, density=1.0)
    s.mouse(anchor, m, (16.25, 6.25), 1000.0)
    n = s.body(DYNAMIC, 20.0, 7.0)
    s.fixture(n, CIRCLE, [0.0, 0.0, 0.5], 1, density=1.0)
    s.mouse(anchor, n, (20.0, 7.5), 6.0, 2.0, 0.3)
    for i in range(6):
        x = _q((-10.0, -4.0, 4.0, 9.0, 16.0, -7.0)[i] + rng.uniform(-0.3, 0.3))
        e = s.body(DYNAMIC, x, _q(16.0 + 2.0 * i + rng.uniform(0.0, 1.0)), angle=_q(rng.uniform(-0.4, 0.4)))
        s.fixture(e, CIRCLE if i % 2 else BOX, [0.0, 0.0, 0.3] if i % 2 else [0.3, 0.3], 1 if i % 2 else 2,
                  density=1.0, friction=0.5)
    return _settings(s, allow_sleep)


def gears(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Gear joints: a motor-driven wheel geared to a larger one (revolute-revolute), a spinning
    pinion geared to a vertical rack on a prismatic joint with limits, two horizontal sliders geared
    together (prismatic-prismatic), and a car whose two wheels are geared to each other through their
    revolute joints on the chassis (bodies C and D of that gear are both the moving chassis); boxes and
    circles fall among them."""
    s = Scene(name="gears")
    g = s.body(STATIC, 0.0, 0.0)
    s.fixture(g, EDGE, [-40.0, 0.0, 40.0, 0.0, 0, 0, 0, 0, 0, 0], friction=0.7)
    w1 = s.body(DYNAMIC, -12.0, 8.0)
    s.fixture(w1, CIRCLE, [0.0, 0.0, 1.0], 1, density=1.0)
    w2 = s.body(DYNAMIC, -8.5, 8.0)
    s.fixture(w2, CIRCLE, [0.0, 0.0, 2.0], 1, density=1.0)
    j0 = s.revolute(g, w1, (-12.0, 8.0), (0.0, 0.0), motor_speed=2.0, max_motor_torque=60.0, flags=2)
    j1 = s.revolute(g, w2, (-8.5, 8.0), (0.0, 0.0))
    s.gear(w1, w2, j0, j1, 2.0)
    # rack and pinion
    p = s.body(DYNAMIC, 2.0, 6.0, w=3.0)
    s.fixture(p, CIRCLE, [0.0, 0.0, 1.0], 1, density=1.0)
    rack = s.body(DYNAMIC, 3.5, 6.0)
    s.fixture(rack, BOX, [0.25, 1.5], 2, density=1.0)
    j3 = s.revolute(g, p, (2.0, 6.0), (0.0, 0.0))
    j4 = s.prismatic(g, rack, (3.5, 6.0), (0.0, 0.0), (0.0, 1.0), lower=-3.0, upper=3.0, flags=1)
    s.gear(p, rack, j3, j4, -1.0)
    # geared sliders on horizontal rails
    s1 = s.body(DYNAMIC, 10.0, 3.0, vx=2.0)
    s.fixture(s1, BOX, [0.5, 0.25], 2, density=1.0)
    s2 = s.body(DYNAMIC, 10.0, 6.0)
    s.fixture(s2, BOX, [0.5, 0.25], 2, density=2.0)
    j6 = s.prismatic(g, s1, (10.0, 3.0), (0.0, 0.0), (1.0, 0.0))
    j7 = s.prismatic(g, s2, (10.0, 6.0), (0.0, 0.0), (1.0, 0.0))
    s.gear(s1, s2, j6, j7, 1.5)
    # a car with geared wheels
    car = s.body(DYNAMIC, 20.0, 3.0, vx=-3.0)
    s.fixture(car, BOX, [1.5, 0.3], 2, density=1.0)
    wa = s.body(DYNAMIC, 19.0, 2.3, vx=-3.0)
    s.fixture(wa, CIRCLE, [0.0, 0.0, 0.5], 1, density=1.0, friction=0.9)
    wb = s.body(DYNAMIC, 21.0, 2.3, vx=-3.0)
    s.fixture(wb, CIRCLE, [0.0, 0.0, 0.5], 1, density=1.0, friction=0.9)
    j9 = s.revolute(car, wa, (-1.0, -0.7), (0.0, 0.0))
    j10 = s.revolute(car, wb, (1.0, -0.7), (0.0, 0.0))
    s.gear(wa, wb, j9, j10, -1.0)
    for i in range(6):
        x = _q((-12.0, -8.5, 2.0, 10.0, 20.0, 3.5)[i] + rng.uniform(-0.3, 0.3))
        e = s.body(DYNAMIC, x, _q(12.0 + 1.5 * i + rng.uniform(0.0, 1.0)), angle=_q(rng.uniform(-0.4, 0.4)))
        s.fixture(e, CIRCLE if i % 2 else BOX, [0.0, 0.0, 0.3] if i % 2 else [0.3, 0.3], 1 if i % 2 else 2,
                  density=1.0, friction=0.5)
    return _settings(s, allow_sleep)


def chain_terrain(rng: SplitMix64, allow_sleep: bool = True) -> Scene:
    """Chain shapes: a static open terrain chain of 40 segments with ghost vertices past both ends, a
    static closed loop holding a few bodies, a kinematic body carrying a zig-zag chain across the
    scene, and circles, boxes and fast bullets (continuous collision against chain children) falling
    onto them."""
    s = Scene(name="chain_terrain")
    g = s.body(STATIC, 0.0, 0.0)
    terrain = [(-40.0 + 2.0 * i, _q(1.2 * math.sin(0.6 * i) + 0.4 * rng.uniform(-1.0, 1.0))) for i in range(41)]
    s.chain(g, terrain, prev=(-42.0, 0.0), next_=(42.0, 0.0), friction=0.6)
    box = s.body(STATIC, 28.0, 10.0, angle=0.1)
    s.chain(box, [(-4.0, -3.0), (4.0, -3.0), (4.0, 3.0), (-4.0, 3.0)], loop=True, friction=0.4)
    for i in range(4):
        b = s.body(DYNAMIC, _q(26.0 + 1.3 * i), _q(10.0 + rng.uniform(-1.0, 1.0)), vx=_q(rng.uniform(-4.0, 4.0)),
                   w=_q(rng.uniform(-2.0, 2.0)))
        s.fixture(b, CIRCLE if i % 2 else BOX, [0.0, 0.0, 0.5] if i % 2 else [0.5, 0.4], 1 if i % 2 else 2,
                  density=1.0, friction=0.3, restitution=0.3)
    k = s.body(KINEMATIC, -12.0, 9.0, vx=1.5, w=0.15)
    s.chain(k, [(-3.0, 0.0), (-1.0, 1.0), (1.0, 0.0), (3.0, 1.0)], friction=0.5)
    for i in range(40):
        x = _q(rng.uniform(-36.0, 22.0))
        y = _q(rng.uniform(5.0, 22.0))
        bullet = i % 10 == 9
        b = s.body(DYNAMIC, x, y, angle=_q(rng.uniform(-1.0, 1.0)), vy=-60.0 if bullet else 0.0,
                   flags=DEFAULT_FLAGS | (8 if bullet else 0))
        if i % 3 == 0:
            s.fixture(b, CIRCLE, [0.0, 0.0, _q(rng.uniform(0.2, 0.6))], 1, density=1.0, friction=0.4)
        else:
            s.fixture(b, BOX, [_q(rng.uniform(0.2, 0.6)), _q(rng.uniform(0.2, 0.6))], 2, density=1.0, friction=0.4)
    return _settings(s, allow_sleep)


# ---------------------------------------------------------------------- named workloads
def config1(allow_sleep: bool = True) -> Scene:
    """210-box pyramid on an edge ground (dt 1/60, 8/3 iterations, 600 steps)."""
    return pyramid(20, allow_sleep=allow_sleep)


def config2(n_bodies: int = 10000, seed: int = 1, allow_sleep: bool = True) -> Scene:
    """Mixed drop into a 200 x 200 m edge box (dt 1/60, 8/3 iterations, 1000 steps)."""
    return drop(n_bodies, SplitMix64(seed), half_size=100.0, allow_sleep=allow_sleep)


def config4(n_worlds: int, first_seed: int, n_bodies: int = 256, allow_sleep: bool = False) -> list:
    """Worlds of the config-2 mix (circles / convex polygons dropped into an edge container), one per
    seed first_seed, first_seed + 1, ...: the scenes the learned warm start is trained and evaluated on.
    n_bodies per world (the full-size mix has 10,000 in a 200 m box; the container here scales with
    the body count as in drop())."""
    return [drop(n_bodies, SplitMix64(first_seed + k), allow_sleep=allow_sleep) for k in range(n_worlds)]


def config3_specs(n_worlds: int = 4096, seed: int = 1, min_bodies: int = 16, max_bodies: int = 512) -> list:
    """The batched workload's worlds as (body count, kind, sub-seed) triples, cheap to draw: the body
    count log-uniform in [min, max], the kind among pyramid (0) / stacks (1) / drop (2)."""
    rng = SplitMix64(seed)
    specs = []
    for _ in range(n_worlds):
        n = int(round(math.exp(rng.uniform(math.log(min_bodies), math.log(max_bodies)))))
        kind = rng.randint(0, 2)
        specs.append((n, kind, rng.next_u64()))
    return specs


def config3_world(spec, allow_sleep: bool = True) -> Scene:
    """One world of the batched workload from its (body count, kind, sub-seed) spec."""
    n, kind, sub_seed = spec
    sub = SplitMix64(sub_seed)
    if kind == 0:
        rows = max(1, int((math.sqrt(8 * n + 1) - 1) // 2))
        return pyramid(rows, allow_sleep=allow_sleep)
    if kind == 1:
        return stacks(n, sub, allow_sleep=allow_sleep)
    return drop(n, sub, allow_sleep=allow_sleep)


def config3(n_worlds: int = 4096, seed: int = 1, allow_sleep: bool = True, min_bodies: int = 16,
            max_bodies: int = 512) -> list:
    """Independent worlds with log-uniform body counts in [min, max] and a seeded kind among
    pyramid / stacks / drop (dt 1/60, 8/3 iterations, 600 steps)."""
    return [config3_world(sp, allow_sleep) for sp in config3_specs(n_worlds, seed, min_bodies, max_bodies)]


def config5(n_bodies: int = 65536, n_chains: int = 512, links: int = 16, half: float = 150.0, seed: int = 1,
            omega: float = 0.05, allow_sleep: bool = True) -> Scene:
    """The joint stress world: a 2*half square container of 4 edges on one kinematic body spinning
    at omega rad/s about the container's centre, holding n_bodies dynamic bodies: n_chains chains of
    `links` revolute-jointed 0.1 x 0.5 m box links (limits +/-30 degrees, no collision inside a
    chain), and loose bodies, 60% boxes (half-extent U[0.2, 0.8]) and 40% circles (radius
    U[0.2, 0.8]). Bodies start on a square grid filling the container, one per cell (cell pitch
    2*half / ceil(sqrt(n_bodies))): a loose body's size is capped at 0.47 of the pitch so none
    overlap (at 65,536 bodies in 300 m the pitch is 1.17 m, so sizes above 0.55 m are capped), and
    each chain fills `links` consecutive cells of a grid column, its joints halfway between cells."""
    rng = SplitMix64(seed)
    s = Scene(name=f"stress{n_bodies}")
    cx, cy = 0.0, half
    k = s.body(KINEMATIC, cx, cy, w=omega)
    for v in ([-half, -half, half, -half], [half, -half, half, half], [half, half, -half, half], [-half, half, -half, -half]):
        s.fixture(k, EDGE, v + [0, 0, 0, 0, 0, 0], friction=0.6)
    g = int(math.ceil(math.sqrt(n_bodies)))
    pitch = 2.0 * half / g
    cap = 0.47 * pitch
    cell = lambda i, j: (_q(cx - half + (i + 0.5) * pitch), _q(cy - half + (j + 0.5) * pitch))
    rows_per_chain = links
    chain_cells = set()
    chains_made = 0
    col, row = 0, 0
    while chains_made < n_chains and col < g:
        if row + rows_per_chain > g:
            col += 2
            row = 0
            continue
        for r in range(rows_per_chain):
            chain_cells.add((col, row + r))
        chains_made += 1
        row += rows_per_chain + 1
    # chains first (bodies then joints per chain), then the loose bodies in grid order
    placed = 0
    made = 0
    col, row = 0, 0
    while made < chains_made:
        if row + rows_per_chain > g:
            col += 2
            row = 0
            continue
        prev = None
        for r in range(rows_per_chain):
            x, y = cell(col, row + rows_per_chain - 1 - r)
            b = s.body(DYNAMIC, x, y)
            s.fixture(b, BOX, [0.1, 0.5], 2, density=1.0, friction=0.4, group=-(made + 1))
            if prev is not None:
                s.revolute(prev, b, (0.0, -0.5 * pitch), (0.0, 0.5 * pitch), 0.0, -math.pi / 6.0, math.pi / 6.0, flags=1)
            prev = b
            placed += 1
        made += 1
        row += rows_per_chain + 1
    for j in range(g):
        for i in range(g):
            if placed >= n_bodies:
                break
            if (i, j) in chain_cells:
                continue
            x, y = cell(i, j)
            size = min(rng.uniform(0.2, 0.8), cap)
            b = s.body(DYNAMIC, x, y, angle=_q(rng.uniform(0.0, 2.0 * math.pi)))
            if rng.uniform() < 0.6:
                s.fixture(b, BOX, [_q(size), _q(size)], 2, density=1.0, friction=0.4)
            else:
                s.fixture(b, CIRCLE, [0.0, 0.0, _q(size)], 1, density=1.0, friction=0.4)
            placed += 1
    return _settings(s, allow_sleep)
