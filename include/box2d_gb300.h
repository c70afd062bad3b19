/*
 * C-ABI of the GB300 Box2D step (libbox2d_gb300.so).
 *
 * The reference Box2D 2.3.2 has no plugin or FFI layer: its boundary is the C++ class API of b2World
 * (Box2D/Dynamics/b2World.h:43-288) with b2Body, b2Fixture, b2Contact and the listener classes. Each
 * entry point below replaces the part of that API named in its comment; the C++ mirror in
 * include/box2d_gb300.hpp (namespace box2d) and the Python package call only these functions.
 *
 * Conventions
 *  - A gb_world handle owns a batch of one or more independent worlds (a single b2World is a batch of
 *    one). World w of the batch is addressed by its index; bodies, fixtures and joints by their
 *    creation index within their world, so index order is creation order.
 *  - Every function returns a gb_status; no function throws or aborts. The library owns all device
 *    memory; the caller owns every host array it passes and keeps it valid for the call only.
 *  - Calls on one handle are not thread-safe (as b2World). Different handles are independent.
 *  - gb_world_step is asynchronous on the handle's CUDA stream; getters and gb_world_sync wait for it.
 */
#ifndef BOX2D_GB300_H
#define BOX2D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int gb_status;
#define GB_OK 0
#define GB_ERR_CAPACITY 1 /* a fixed-capacity device buffer overflowed during a step */
#define GB_ERR_TIMEOUT 2  /* a bounded device loop (TOI sub-steps) hit its limit */
#define GB_ERR_INVALID 3  /* bad argument, or a call made while the world is locked */
#define GB_ERR_CUDA 4     /* a CUDA runtime call failed (no device, launch error, ...) */

typedef struct gb_world gb_world;
typedef struct gb_mlp gb_mlp;

/* b2World settings (b2World::b2World(gravity), SetAllowSleeping, SetWarmStarting,
 * SetContinuousPhysics, SetSubStepping: Box2D/Dynamics/b2World.h:48,145-217). */
typedef struct gb_world_def {
    float gravity_x, gravity_y;
    int allow_sleep;
    int warm_starting;
    int continuous_physics;
    int sub_stepping;
} gb_world_def;

/* b2World::SetGravity, SetAllowSleeping, SetWarmStarting, SetContinuousPhysics, SetSubStepping and
 * SetAutoClearForces (Box2D/Dynamics/b2World.h:145-217, b2World.cpp:370-385) of world w between
 * steps: def holds the new settings; turning allow_sleep off wakes every body (b2Body::SetAwake(true));
 * auto_clear_forces 0 keeps each body's force and torque after a step (cleared by
 * gb_world_clear_forces, b2World::ClearForces, Box2D/Dynamics/b2World.cpp:967-974). */
gb_status gb_world_set_settings(gb_world* world, int w, const gb_world_def* def, int auto_clear_forces);
gb_status gb_world_clear_forces(gb_world* world, int w);

/* b2World::b2World (Box2D/Dynamics/b2World.cpp:34) for n_worlds independent worlds. */
gb_status gb_world_create(int n_worlds, const gb_world_def* defs, gb_world** out);
/* b2World::~b2World (Box2D/Dynamics/b2World.cpp:58) */
gb_status gb_world_destroy(gb_world* world);

/* b2World::CreateBody (Box2D/Dynamics/b2World.cpp:96). Per body: type (0 static, 1 kinematic,
 * 2 dynamic); f[9] = position.x, position.y, angle, linearVelocity.x, .y, angularVelocity,
 * linearDamping, angularDamping, gravityScale; flags: 1 allowSleep, 2 awake, 4 fixedRotation,
 * 8 bullet, 16 active. out_ids (optional) receives the new body indices. */
gb_status gb_create_bodies(gb_world* world, int w, int n, const int* type, const float* f, const int* flags,
                           int* out_ids);

/* b2Body::CreateFixture (Box2D/Dynamics/b2Body.cpp:151). Per fixture: body index; shape type
 * 0 circle {p.x, p.y, radius}, 1 edge {v1.x, v1.y, v2.x, v2.y, v0.x, v0.y, v3.x, v3.y, hasV0, hasV3,
 * chain} (chain 0 for a b2EdgeShape; 1 and 2 for the first and each next child of a chain, as
 * gb_create_chain writes them: a child's box has no radius, b2ChainShape.cpp:171-187),
 * 2 polygon from n points (b2PolygonShape::Set), 3 box {hx, hy} or, with n == 5, {hx, hy, center.x,
 * center.y, angle} (b2PolygonShape::SetAsBox); shape[16] per fixture; mat[3] = density, friction,
 * restitution; filt[4] = categoryBits, maskBits, groupIndex, isSensor. */
gb_status gb_create_fixtures(gb_world* world, int w, int n, const int* body, const int* shape_type,
                             const float* shape, const int* shape_n, const float* mat, const int* filt,
                             int* out_ids);

/* b2ChainShape::CreateChain or CreateLoop + b2Body::CreateFixture (Box2D/Collision/Shapes/
 * b2ChainShape.cpp:36-80, Box2D/Dynamics/b2Fixture.cpp:121-137): count vertices xy[2 * count] make
 * count - 1 child edges (a loop, loop != 0, closes with a count-th), each with its ghost vertices as
 * b2ChainShape::GetChildEdge gives them, created as consecutive fixtures from *first_id on; the
 * fixture ids that contacts, events and queries report for the chain are first_id + child index.
 * An open chain's SetPrevVertex / SetNextVertex: prev_next = {prev.x, prev.y, next.x, next.y} with
 * ghost_flags bit 0 / bit 1. mat and filt as gb_create_fixtures, shared by the children. */
gb_status gb_create_chain(gb_world* world, int w, int body, const float* xy, int count, int loop,
                          const float* prev_next, int ghost_flags, const float* mat, const int* filt, int* first_id);

/* b2World::CreateJoint with a b2RevoluteJointDef (Box2D/Dynamics/b2World.cpp:185,
 * Box2D/Dynamics/Joints/b2RevoluteJoint.h:36). f[9] = localAnchorA.x, .y, localAnchorB.x, .y,
 * referenceAngle, lowerAngle, upperAngle, motorSpeed, maxMotorTorque; flags: 1 enableLimit,
 * 2 enableMotor, 4 collideConnected. */
gb_status gb_create_revolute_joints(gb_world* world, int w, int n, const int* body_a, const int* body_b,
                                    const float* f, const int* flags, int* out_ids);

/* b2World::CreateJoint for the joint definitions built here (Box2D/Dynamics/b2World.cpp:185;
 * Box2D/Dynamics/Joints/b2RevoluteJoint.h:36, b2DistanceJoint.h:30, b2WeldJoint.h:28,
 * b2PrismaticJoint.h:30, b2WheelJoint.h:30, b2RopeJoint.h:28, b2FrictionJoint.h:25,
 * b2MotorJoint.h:26, b2MouseJoint.h:24, b2PulleyJoint.h:26, b2GearJoint.h:24). type: GB_JOINT_*. f[GB_JOINT_FLOATS] per joint (the fields of the definition;
 * anchors and axes in body-local coordinates):
 *   revolute   localAnchorA.x, .y, localAnchorB.x, .y, referenceAngle, lowerAngle, upperAngle,
 *              motorSpeed, maxMotorTorque (as gb_create_revolute_joints)
 *   distance   localAnchorA.x, .y, localAnchorB.x, .y, length, frequencyHz, dampingRatio
 *   weld       localAnchorA.x, .y, localAnchorB.x, .y, referenceAngle, frequencyHz, dampingRatio
 *   prismatic  localAnchorA.x, .y, localAnchorB.x, .y, localAxisA.x, .y (normalised as the
 *              reference's constructor does), referenceAngle, lowerTranslation, upperTranslation,
 *              maxMotorForce, motorSpeed
 *   wheel      localAnchorA.x, .y, localAnchorB.x, .y, localAxisA.x, .y (taken as given, as the
 *              reference does), maxMotorTorque, motorSpeed, frequencyHz, dampingRatio
 *   rope       localAnchorA.x, .y, localAnchorB.x, .y, maxLength
 *   friction   localAnchorA.x, .y, localAnchorB.x, .y, maxForce, maxTorque
 *   motor      linearOffset.x, .y, angularOffset, maxForce, maxTorque, correctionFactor
 *   mouse      target.x, .y (world; body B's local anchor is the target's point on B at creation),
 *              maxForce, frequencyHz, dampingRatio (body A is normally a static body)
 *   pulley     groundAnchorA.x, .y, groundAnchorB.x, .y (world), localAnchorA.x, .y, localAnchorB.x,
 *              .y, lengthA, lengthB, ratio (non-zero)
 *   gear       joint1, joint2 (indices of revolute or prismatic joints of the same world, as exact
 *              floats), ratio; a and b are the definition's bodyA/bodyB (contact filtering only:
 *              the joint acts on joint1's and joint2's body B, b2GearJoint.cpp:49-136)
 * Unused trailing floats are ignored. flags: 1 enableLimit (revolute, prismatic), 2 enableMotor
 * (revolute, prismatic, wheel), 4 collideConnected. */
#define GB_JOINT_REVOLUTE 0
#define GB_JOINT_DISTANCE 1
#define GB_JOINT_WELD 2
#define GB_JOINT_PRISMATIC 3
#define GB_JOINT_WHEEL 4
#define GB_JOINT_ROPE 5
#define GB_JOINT_FRICTION 6
#define GB_JOINT_MOTOR 7
#define GB_JOINT_MOUSE 8
#define GB_JOINT_PULLEY 9
#define GB_JOINT_GEAR 10
#define GB_JOINT_FLOATS 12
gb_status gb_create_joints(gb_world* world, int w, int n, const int* type, const int* body_a, const int* body_b,
                           const float* f, const int* flags, int* out_ids);

/* Bulk scene build into world w: body b is created, then every fixture whose fix_body == b (the array
 * is sorted by body), then all joints (joint_type NULL: all revolute), GB_JOINT_FLOATS floats each as
 * gb_create_joints. Equivalent to the calls above interleaved. */
gb_status gb_build_world(gb_world* world, int w, int nb, const int* body_type, const float* body_f,
                         const int* body_flags, int nf, const int* fix_body, const int* fix_type,
                         const float* fix_shape, const int* fix_n, const float* fix_mat, const int* fix_filt,
                         int nj, const int* joint_type, const int* joint_a, const int* joint_b, const float* joint_f,
                         const int* joint_flags);

/* Copies host-side changes (new bodies, fixtures, joints) to device memory. gb_world_step does this
 * implicitly when needed; calling it explicitly moves the upload out of the first step. */
gb_status gb_world_upload(gb_world* world);

/* b2World::Step (Box2D/Dynamics/b2World.cpp:888): one step of every world of the batch, queued on
 * the handle's stream. Listener events are recorded on the device when enabled. */
gb_status gb_world_step(gb_world* world, float dt, int velocity_iterations, int position_iterations);

/* Waits for queued steps and returns the first error any world raised since the last sync. */
/* World checkpoints (the reference has only b2World::Dump, Box2D/Dynamics/b2World.cpp:1271-1328,
 * which prints code that rebuilds the scene without its contacts): gb_world_checkpoint writes world
 * w's whole state between steps (bodies with their sweeps, sleep times and forces; fixtures, proxies
 * and the tree's free list; joints with their impulses; the contact list in order with manifolds and
 * impulses; the world's settings; the broadphase tree when the handle tracks it) to buf and puts the
 * byte count in *size (buf NULL: only the count; cap too small: GB_ERR_CAPACITY). gb_world_restore
 * replaces world w of any handle with such a checkpoint; the steps that follow are bit for bit those
 * of the world it was taken from (under the same solver settings). A checkpoint restores only into
 * a library of the same build layout (GB_ERR_INVALID otherwise, and for malformed data). */
gb_status gb_world_checkpoint(gb_world* world, int w, void* buf, size_t cap, size_t* size);
gb_status gb_world_restore(gb_world* world, int w, const void* buf, size_t size);

/* b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality (Box2D/Dynamics/b2World.cpp:1246-1259):
 * the height, the largest child height difference and the node-perimeter ratio of the reference
 * broadphase's dynamic tree. The device step keeps no tree (its pair finding works on the fat boxes),
 * so a handle that answers these keeps one on the host: gb_world_track_tree(world, 1), before any
 * fixture with a proxy exists in any of its worlds (GB_ERR_INVALID after), has every world replay
 * the tree's history: the proxies created and destroyed between steps, and every fat box the device
 * gives a proxy, which the step logs. A tracking handle replays the previous step's log before each
 * step, which waits for that step. gb_world_tree_stats reads world w's three values (any pointer may be
 * NULL); GB_ERR_INVALID when the handle does not track, GB_ERR_CAPACITY when a world's log ran out of
 * room (more than 8 re-insertions per proxy plus 256 between two replays). */
gb_status gb_world_track_tree(gb_world* world, int on);
gb_status gb_world_tree_stats(gb_world* world, int w, int* height, int* balance, float* quality);

/* b2Body property changes between steps (no step in progress): prop GB_BODY_TYPE (v[0] 0 static,
 * 1 kinematic, 2 dynamic; b2Body::SetType, Box2D/Dynamics/b2Body.cpp:115-166: mass reset, a static
 * body's velocities zeroed and fixtures synchronised, the body woken, its force cleared, its contacts
 * destroyed and its proxies queried again at the next step), GB_BODY_ACTIVE (v[0] != 0; SetActive,
 * :456-499: proxies created in the fixture list's order, or destroyed with the contacts),
 * GB_BODY_FIXED_ROTATION (SetFixedRotation, :501-520), GB_BODY_BULLET, GB_BODY_SLEEPING_ALLOWED
 * (turning it off wakes the body), GB_BODY_LINEAR_DAMPING, GB_BODY_ANGULAR_DAMPING,
 * GB_BODY_GRAVITY_SCALE (v[0]; b2Body.h:593-682), GB_BODY_MASS_DATA (SetMassData, :355-394: v[0] mass,
 * v[1..2] center, v[3] inertia about the body origin; dynamic bodies only), GB_BODY_RESET_MASS_DATA
 * (ResetMassData, :283-353; v unused). calls (optional, cap records of 3 ints, *n_calls
 * the count) receives the EndContact calls {2, fixtureA, fixtureB} of the contacts it destroys. */
#define GB_BODY_TYPE 0
#define GB_BODY_ACTIVE 1
#define GB_BODY_FIXED_ROTATION 2
#define GB_BODY_BULLET 3
#define GB_BODY_SLEEPING_ALLOWED 4
#define GB_BODY_LINEAR_DAMPING 5
#define GB_BODY_ANGULAR_DAMPING 6
#define GB_BODY_GRAVITY_SCALE 7
#define GB_BODY_MASS_DATA 8
#define GB_BODY_RESET_MASS_DATA 9
gb_status gb_body_set(gb_world* world, int w, int body, int prop, const float* v, int* calls, int cap, int* n_calls);

/* Joint changes between steps (no step in progress), with the reference's wakes of both bodies and
 * resets of the limit impulse: GB_JOINT_MOTOR_SPEED, GB_JOINT_MAX_MOTOR (torque; a prismatic joint's
 * force), GB_JOINT_ENABLE_MOTOR (revolute, prismatic, wheel: b2RevoluteJoint.cpp:419-443,
 * b2PrismaticJoint.cpp:585-604, b2WheelJoint.cpp:377-396); GB_JOINT_ENABLE_LIMIT, GB_JOINT_LIMITS
 * (v[0] lower <= v[1] upper; revolute, prismatic: b2RevoluteJoint.cpp:450-483,
 * b2PrismaticJoint.cpp:546-577); GB_JOINT_LENGTH (distance); GB_JOINT_FREQUENCY,
 * GB_JOINT_DAMPING_RATIO (distance, weld, the wheel's spring, mouse); GB_JOINT_MAX_LENGTH (rope);
 * GB_JOINT_MAX_FORCE (friction, motor, mouse); GB_JOINT_MAX_TORQUE (friction, motor);
 * GB_JOINT_LINEAR_OFFSET (v[0..1]), GB_JOINT_ANGULAR_OFFSET, GB_JOINT_CORRECTION_FACTOR (motor,
 * b2MotorJoint.cpp:228-284); GB_JOINT_RATIO (gear). A property the joint's type does not have
 * returns GB_ERR_INVALID. */
#define GB_JOINT_MOTOR_SPEED 0
#define GB_JOINT_MAX_MOTOR 1
#define GB_JOINT_ENABLE_MOTOR 2
#define GB_JOINT_ENABLE_LIMIT 3
#define GB_JOINT_LIMITS 4
#define GB_JOINT_LENGTH 5
#define GB_JOINT_FREQUENCY 6
#define GB_JOINT_DAMPING_RATIO 7
#define GB_JOINT_MAX_LENGTH 8
#define GB_JOINT_MAX_FORCE 9
#define GB_JOINT_MAX_TORQUE 10
#define GB_JOINT_LINEAR_OFFSET 11
#define GB_JOINT_ANGULAR_OFFSET 12
#define GB_JOINT_CORRECTION_FACTOR 13
#define GB_JOINT_RATIO 14
gb_status gb_joint_set(gb_world* world, int w, int joint, int prop, const float* v);

/* b2Joint::GetReactionForce(inv_dt) and GetReactionTorque(inv_dt) of any joint type
 * (Box2D/Dynamics/Joints/*.cpp) after the last step: out[0..1] the force on body B at the anchor,
 * out[2] the torque. Waits for the step in flight. */
gb_status gb_get_joint_reaction(gb_world* world, int w, int joint, float inv_dt, float* out);

/* b2Fixture::TestPoint (op 0: in[0..1] the point; out[0] 1 when inside), RayCast (op 1: in[0..1] p1,
 * in[2..3] p2, in[4] maxFraction; out = hit, normal x, y, fraction), GetAABB (op 2: out = lower x,
 * y, upper x, y) and GetMassData (op 3: out = mass, center x, y, inertia about the body origin) of a
 * fixture (a chain child by its own index) at the body's current transform
 * (Box2D/Dynamics/b2Fixture.h:313-342). Waits for the step in flight. */
gb_status gb_fixture_query(gb_world* world, int w, int fixture, int op, const float* in, float* out);

/* b2PolygonShape::Set (mode 0: in = n points x, y; Box2D/Collision/Shapes/b2PolygonShape.cpp:119-252,
 * the hull of welded points), SetAsBox(hx, hy) (mode 1: in = hx, hy) and SetAsBox(hx, hy, center,
 * angle) (mode 2: in = hx, hy, cx, cy, angle; :47-70): out = centroid (2), vertices (8 x 2), normals
 * (8 x 2), *count the vertices, as the library stores the shape. No device work. */
gb_status gb_polygon_shape(int mode, const float* in, int n, float* out, int* count);

/* b2World::ShiftOrigin (Box2D/Dynamics/b2World.cpp:1261-1282) of world w between steps: bodies, the
 * mouse joints' targets, the pulleys' ground anchors and the broadphase's boxes move by -(x, y). */
gb_status gb_world_shift_origin(gb_world* world, int w, float x, float y);

/* b2Fixture changes between steps (no step in progress): prop GB_FIXTURE_FRICTION, GB_FIXTURE_RESTITUTION
 * (v[0]; b2Fixture::SetFriction, SetRestitution, Box2D/Dynamics/b2Fixture.h:300-340: new contacts mix
 * the new value, existing ones keep theirs, as in the reference), GB_FIXTURE_DENSITY (v[0] >= 0;
 * SetDensity: the body's mass follows at its next mass reset), GB_FIXTURE_SENSOR (v[0] != 0;
 * SetSensor, b2Fixture.cpp:418-425: a change wakes the body), GB_FIXTURE_FILTER (v[0] category,
 * v[1] mask, v[2] group; SetFilterData, b2Fixture.cpp:181-214: the fixture's contacts are filtered
 * again at the next step and its proxies look for new pairs). A chain is addressed by its first
 * child's index and changes as a whole. */
#define GB_FIXTURE_FRICTION 0
#define GB_FIXTURE_RESTITUTION 1
#define GB_FIXTURE_DENSITY 2
#define GB_FIXTURE_SENSOR 3
#define GB_FIXTURE_FILTER 4
gb_status gb_fixture_set(gb_world* world, int w, int fixture, int prop, const float* v);

/* b2Body::GetMass, GetInertia (about the body origin), GetLocalCenter, GetLinearDamping,
 * GetAngularDamping, GetGravityScale (Box2D/Dynamics/b2Body.h:227-260, 546-556, 593-682) into
 * out[0..6]; *flags (optional) = GetType() | 4 IsBullet | 8 IsFixedRotation | 16 IsSleepingAllowed
 * | 32 IsActive. None of these change during a step, so no device read is made. */
gb_status gb_get_body_info(gb_world* world, int w, int body, float* out, int* flags);

/* b2World::DestroyBody (Box2D/Dynamics/b2World.cpp:133), b2World::DestroyJoint (:274) and
 * b2Body::DestroyFixture (Box2D/Dynamics/b2Body.cpp:216), between steps, with the reference's order of
 * effects: a body's joints (each announced to the destruction listener, then destroyed: both bodies
 * woken, contacts between them flagged for filtering unless the joint let them collide), its contacts
 * (EndContact when touching; both bodies woken when the manifold had points), its fixtures (each
 * announced) and their broadphase proxies; a fixture's contacts and proxies, then the body's mass data
 * reset. A chain fixture is destroyed by its first child's id, with all its children. Indices of other
 * bodies, fixtures and joints do not change; a destroyed body reads back as zeros, and bodies created
 * later take the next indices. Proxy ids of later fixtures reuse the freed tree nodes exactly as the
 * reference's b2DynamicTree does. The listener calls go to calls (3 ints each, at most cap):
 * {0, joint, 0} SayGoodbye(b2Joint*), {1, fixture, 0} SayGoodbye(b2Fixture*), {2, fixtureA, fixtureB}
 * EndContact; n_calls receives their number. GB_ERR_INVALID for an index that is out of range or
 * already destroyed. */
gb_status gb_destroy_body(gb_world* world, int w, int body, int* calls, int cap, int* n_calls);
gb_status gb_destroy_joint(gb_world* world, int w, int joint, int* calls, int cap, int* n_calls);
gb_status gb_destroy_fixture(gb_world* world, int w, int fixture, int* calls, int cap, int* n_calls);

/* A step split at its collide phase, for a b2ContactListener::PreSolve that changes contacts
 * (Box2D/Dynamics/b2WorldCallbacks.h:105-120; b2Contact::SetEnabled, SetFriction, SetRestitution,
 * SetTangentSpeed, Contacts/b2Contact.h:98-152), with one synchronisation: gb_world_step_begin runs
 * b2World::Step up to and including b2ContactManager::Collide (new-fixture pairs, narrowphase,
 * Begin/End/PreSolve calls recorded, gb_world_read_events reads them); gb_contact_edits then applies
 * the listener's changes, in order: edit.contact is the contact's position in the world's contact
 * list (gb_get_contacts order at this point), flags bit 0 sets the enabled flag to edit.enabled, bit 1
 * the friction, bit 2 the restitution, bit 3 the tangent speed; gb_world_step_end runs the rest of the
 * step (islands, solver, continuous phase). The world is locked between the two (creation and
 * destruction return GB_ERR_INVALID) and gb_world_step / gb_world_graph_step are refused. The
 * continuous phase's own PreSolve calls (contacts with a static, kinematic or bullet body updated at
 * a time of impact) stay notifications: the split is exact for listeners that change only other
 * contacts. */
typedef struct gb_contact_edit {
    int world, contact, flags, enabled;
    float friction, restitution, tangent_speed, reserved;
} gb_contact_edit;
gb_status gb_world_step_begin(gb_world* world, float dt, int velocity_iterations, int position_iterations);
gb_status gb_contact_edits(gb_world* world, int n, const gb_contact_edit* edits);
gb_status gb_world_step_end(gb_world* world);

/* b2World::SetContactFilter (Box2D/Dynamics/b2World.cpp:94, b2ContactFilter in b2WorldCallbacks.h:
 * 52-63): should_collide(user, world, fixtureA, fixtureB) decides, in place of the default
 * category/mask/group filter, whether the fixtures of a new pair get a contact (b2ContactManager::
 * AddPair) and whether a contact flagged for filtering survives (b2ContactManager::Collide), with the
 * reference's ordered fixture pair; nonzero means collide. The verdicts are kept per ordered pair and
 * asked once: the device uses the default filter's verdict for a pair it meets first, the library asks
 * the callback after the step, and when an answer differs it restores the state from before the step
 * (a copy of every device column, kept while a filter is set) and runs the step again, so every step
 * equals the reference's. Steps with a filter are therefore synchronous (the callback runs on the
 * calling thread inside gb_world_step), gb_world_graph_step runs plain steps, and the split step is
 * refused. gb_world_refilter forgets a fixture's verdicts (b2Fixture::Refilter; flag its contacts with
 * a filter change too). gb_world_filter_stats: steps run again so far and verdicts kept. fn == NULL
 * restores the default filter. At most 2^20 fixtures per world. */
typedef int (*gb_should_collide_fn)(void* user, int world, int fixture_a, int fixture_b);
gb_status gb_world_set_contact_filter(gb_world* world, gb_should_collide_fn fn, void* user);
gb_status gb_world_refilter(gb_world* world, int w, int fixture);
gb_status gb_world_filter_stats(gb_world* world, long long* replays, int* verdicts);

gb_status gb_world_sync(gb_world* world);

/* Grow-and-retry: with attempts > 0 every gb_world_step (and gb_world_graph_step, which then does not
 * replay a graph) keeps a copy of the device state, waits for the step, and when a world overflowed a
 * fixed buffer (contact slots, pairs, island rows: GB_ERR_CAPACITY) or reached the time-of-impact
 * event limit (GB_ERR_TIMEOUT) puts the state back, doubles that world's contact capacity (or the
 * event limit) and runs the step again, up to `attempts` times; the step's result is then the one the
 * reference takes. Each step waits for the device; not for steps captured into a caller's graph.
 * gb_world_recoveries: the steps run again so far. */
gb_status gb_world_set_recovery(gb_world* world, int attempts);
gb_status gb_world_recoveries(gb_world* world, long long* retries);

/* No counterpart in the reference (whose buffers grow on demand). The fixed capacities of the device
 * step, for callers that size memory themselves and for tests of the error paths: contact_capacity
 * > 0 sets the contact slots of each world at its first upload (0 keeps the default, max(64, 8 x
 * fixtures); GB_ERR_INVALID once the world is on the device); max_toi_events bounds the
 * time-of-impact events of each world in one step (default 4096). A step that needs more contact
 * slots than it has, or more events, stops that work, completes the step and makes the next
 * gb_world_sync return GB_ERR_CAPACITY or GB_ERR_TIMEOUT; the world's state after such a step is not
 * the reference's and the world should be rebuilt (gb_world_destroy, then create it again with larger
 * limits). Every loop on the device is bounded, so the error never stalls the GPU. */
gb_status gb_world_set_limits(gb_world* world, int contact_capacity, int max_toi_events);

/* Island solver of the following steps. GB_SOLVER_PLAIN (default) is b2Island::Solve's sequential
 * per-island Gauss-Seidel order (Box2D/Dynamics/b2Island.cpp:185-384), bit-exact with the reference.
 * GB_SOLVER_COLOURED solves the same contact constraints colour by colour (constraints of one colour
 * share no dynamic body and are solved in parallel); it converges like Gauss-Seidel but its results
 * are not the reference's bits. tolerance > 0 ends the velocity iterations of a world (plain: of an
 * island) once its velocity residual is at most tolerance (m/s); velocity_iterations stays the
 * maximum. measure_residual != 0 records each world's velocity residual after the velocity
 * iterations (gb_world_solver_stats). The velocity residual is the largest over contact points of
 * the natural-map residual of the contact conditions in velocity units: |ni - max(0, ni - mn (vn -
 * bias))| / mn for the normal impulse ni (effective mass mn) and |ti - clamp(ti - mt vt, -mu ni,
 * mu ni)| / mt for the tangent impulse ti; it is |vn - bias| on active normal points, |vt| on friction
 * strictly inside its cone, and zero exactly at a solution. */
#define GB_SOLVER_PLAIN 0
#define GB_SOLVER_COLOURED 1
gb_status gb_world_set_solver(gb_world* world, int solver, float tolerance, int measure_residual);

/* Per world of the last step (arrays of n_worlds, each may be NULL): colours used by the coloured
 * solver, velocity iterations run, velocity residual (when measured). */
gb_status gb_world_solver_stats(gb_world* world, int* colours, int* vel_iters, float* residual);

/* Launch plan of the step (no counterpart in the reference, which steps one world on one thread).
 * Worlds are scheduled largest first (by fixture count) and split into up to 4 classes, contiguous
 * ranges of that schedule; each class is one launch with one CTA per world, its own CTA size and
 * shared-memory shape, the launches forked onto side streams and joined back to the handle's stream.
 * Every plan computes identical results; plans differ only in speed.
 * gb_world_autotune arms the online autotuner: the next steps_per_candidate x (number of candidate
 * plans) calls of gb_world_step run the candidates in turn, one step each per round (they are real
 * steps), timed with CUDA events; then the candidate with the smallest median time becomes the plan.
 * Tuning is skipped while the stream is being captured.
 * gb_world_launch_plan reports the plan, classes[5 * i] = first schedule slot, count, threads per
 * CTA, shared-memory island rows, shared-memory contacts, and after tuning the best time (ms) each
 * candidate took. gb_world_set_launch_plan sets a plan in the same layout (classes must cover the
 * schedule in order; threads a multiple of 32 in [32, 512], the continuous phase using at most 64
 * of them; at most 48 KB of shared memory). */
gb_status gb_world_autotune(gb_world* world, int steps_per_candidate);
/* gb_world_step as a CUDA graph: the first call (and any call after the step's parameters, solver
 * or plan changed, or device memory was reallocated) captures one step, every launch of the plan,
 * from the handle's stream into a graph; every call launches that graph once on the stream. */
gb_status gb_world_graph_step(gb_world* world, float dt, int velocity_iterations, int position_iterations);
gb_status gb_world_launch_plan(gb_world* world, int* classes, int cap, int* n_classes, float* candidate_ms,
                               int ms_cap, int* n_candidates);
gb_status gb_world_set_launch_plan(gb_world* world, const int* classes, int n);

/* Per world of the last step (array of n_worlds): the deepest contact penetration (m) the position
 * solver started from, i.e. minus the smallest separation of its first iteration (0 when none). */
gb_status gb_world_contact_stats(gb_world* world, float* max_penetration);

/* Binds the handle to a caller-owned cudaStream_t (NULL = the handle's own stream). */
gb_status gb_world_set_stream(gb_world* world, void* cuda_stream);

/* b2ContactListener (Box2D/Dynamics/b2WorldCallbacks.h:84-130) as a device event log. With events
 * on, every step records, per world and in the reference's call order, the listener calls
 * b2World::Step would make: records[4] = kind (0 BeginContact, 1 EndContact, 2 PreSolve,
 * 3 PostSolve), fixtureA, fixtureB, and for a PostSolve b2ContactImpulse::count; impulses[4] = the
 * PostSolve's normal impulses 0, 1 and tangent impulses 0, 1 (zero otherwise). Order: the collide phase in contact-list order
 * (Update's Begin/End then PreSolve, or Destroy's End), then PostSolve per solved island in island
 * order, then the continuous phase's calls in event order. gb_world_set_events(1) reallocates the
 * device columns (the state is kept); gb_world_read_events reads the last step's records of world w
 * (up to cap; *n receives the count) and returns GB_ERR_CAPACITY if the log overflowed. PreSolve is
 * recorded as a notification: a listener sees it after the step and cannot change the contact. */
gb_status gb_world_set_events(gb_world* world, int enable);
gb_status gb_world_read_events(gb_world* world, int w, int* records, float* impulses, int cap, int* n);

/* World queries on the device (b2World::QueryAABB, b2World::RayCast: Box2D/Dynamics/b2World.h:116-124,
 * b2World.cpp:965-1020), run after the queued steps. gb_world_query_aabb: for n boxes aabbs[4] =
 * lower.x, lower.y, upper.x, upper.y, the fixtures whose broadphase fat AABB overlaps the box (the
 * leaves b2DynamicTree::Query reports), in fixture order: query i's fixtures are
 * fixtures[offsets[i] .. offsets[i + 1]) (offsets has n + 1 entries); *total receives the number of
 * results, GB_ERR_CAPACITY when it exceeds cap (offsets stay valid). gb_world_raycast: for n segments
 * rays[4] = p1.x, p1.y, p2.x, p2.y, the closest hit as a callback that returns each reported
 * fraction gets it: fixture[i] (-1 when none), hit[5] = fraction, point.x, point.y, normal.x,
 * normal.y (b2RayCastOutput and the reported point); equal fractions resolve to the lowest fixture
 * index (the reference keeps the last one its tree traversal reports). Sensors are included. */
gb_status gb_world_query_aabb(gb_world* world, int w, int n, const float* aabbs, int* offsets, int* fixtures, int cap,
                             int* total);
gb_status gb_world_raycast(gb_world* world, int w, int n, const float* rays, int* fixture, float* hit);
/* Every fixture the segment ray[4] = p1.x, p1.y, p2.x, p2.y hits (b2Fixture::RayCast with maxFraction
 * 1, Box2D/Dynamics/b2Fixture.h:308-311), the material b2World::RayCast's callback loop needs
 * (Box2D/Dynamics/b2World.cpp:1021-1035): fixtures[k] and hits[5 k] = fraction, point.x, point.y,
 * normal.x, normal.y, in fixture order (the reference's order is its tree's), at most cap; *n receives
 * the number of hits, GB_ERR_CAPACITY when it exceeds cap. A caller replays its callback over them,
 * skipping hits beyond the fraction the callback has clipped the ray to. */
gb_status gb_world_raycast_all(gb_world* world, int w, const float* ray, int* fixtures, float* hits, int cap, int* n);
/* b2World::GetProfile (Box2D/Dynamics/b2World.h:196, b2Profile in b2TimeStep.h:27-37) of world w's
 * last step in milliseconds at the GPU's SM clock: ms[8] = step, collide, solve, solveInit,
 * solveVelocity, solvePosition, broadphase, solveTOI (the flat narrowphase and time-of-impact
 * pre-passes over all worlds are not in any world's figure). */
gb_status gb_world_get_profile(gb_world* world, int w, float* ms);

/* Counts (b2World::GetBodyCount, GetContactCount, GetProxyCount: b2World.h:160-170). */
gb_status gb_world_counts(gb_world* world, int w, int* bodies, int* fixtures, int* contacts, int* joints);

/* Body state read-back in creation order, 12 floats per body: transform p.x, p.y, sweep angle a,
 * world center c.x, c.y, linearVelocity.x, .y, angularVelocity, transform q.s, q.c, sleepTime,
 * awake (0/1) (b2Body::GetPosition, GetAngle, GetWorldCenter, GetLinearVelocity,
 * GetAngularVelocity, GetTransform, IsAwake: Box2D/Dynamics/b2Body.h). */
gb_status gb_get_bodies(gb_world* world, int w, float* out);

/* Contacts of world w in b2World::GetContactList order (b2World.h:124). ints[8] per contact:
 * fixtureA, fixtureB, flags (b2Contact e_* bits), pointCount, manifold type, id0, id1, toiCount;
 * floats[12]: localNormal.xy, localPoint.xy, then per point localPoint.xy, normalImpulse,
 * tangentImpulse (b2Contact::GetManifold). *count receives the number of contacts (may exceed cap). */
gb_status gb_get_contacts(gb_world* world, int w, int* ints, float* floats, int cap, int* count);

/* Broadphase proxies per fixture: proxy id (b2FixtureProxy::proxyId) and fat AABB
 * (b2BroadPhase::GetFatAABB, Box2D/Collision/b2BroadPhase.h:107). */
gb_status gb_get_proxies(gb_world* world, int w, int* proxy_ids, float* fat_aabbs);

/* Per-world diagnostics of the last step: islands solved, TOI sub-steps. */
gb_status gb_world_stats(gb_world* world, int w, int* islands, int* toi_events);

/* Batch totals over all worlds after the last step, out[8] = live contacts, bodies solved in
 * islands, contacts solved in islands, broadphase pairs produced, islands, TOI sub-steps, proxies,
 * dynamic bodies. */
gb_status gb_world_totals(gb_world* world, long long* out);

/* Per-world SM clock cycles spent in the phases of the last step (the device counterpart of
 * b2World::GetProfile, Box2D/Dynamics/b2World.h:196, b2Profile in b2TimeStep.h:27-37):
 * out[GB_PROFILE_SLOTS * w + i] for i = 0 new-fixture pairs, 1 collide, 2 island build, 3 island
 * solve, 4 fixture sync, 5 pairs, 6 continuous (TOI), 7 whole step; the island solve split 8
 * integrate + constraint init, 9 warm start + velocity sweeps, 10 impulses + position integration,
 * 11 position sweeps, 12 write-back, 13 sleep; 14 broadphase pair finding and sorting, 15 contact
 * creation; the continuous split 16 classification + time of impact, 17 earliest-event selection,
 * 18 event mini-island build, 19 mini-island solve, 20 fixture sync + contact invalidation,
 * 21 pair finding after events; the coloured solver's island build split 22 components and keys,
 * 23 key sort (zero for the plain solver). The narrowphase and time-of-impact pre-passes run
 * flat over all worlds' contacts before the collide and continuous phases and are not counted. */
#define GB_PROFILE_SLOTS 24
gb_status gb_world_profile(gb_world* world, unsigned long long* out);

/* One b2World::Step of every world (a real step, with the current plan, not from the captured
 * graph), timed stage by stage with CUDA events on the handle's stream: ms[0] the narrowphase
 * pre-pass, ms[1] the per-world step up to the continuous phase (every class), ms[2] the
 * time-of-impact pre-pass, ms[3] the per-world continuous phase (every class). The whole-batch
 * counterpart of b2World::GetProfile's step timings (Box2D/Dynamics/b2World.h:196, b2Profile in
 * b2TimeStep.h:27-37); blocks until the step is done. */
gb_status gb_world_stage_times(gb_world* world, float dt, int velocity_iterations, int position_iterations,
                               float* ms);

/* b2Body state changes between steps, each with the reference method's semantics (Box2D/Dynamics/
 * b2Body.cpp:419-441 SetTransform; b2Body.h:501-530 SetLinearVelocity, SetAngularVelocity; 635-655
 * SetAwake; 739-830 ApplyForce, ApplyForceToCenter, ApplyTorque, ApplyLinearImpulse,
 * ApplyAngularImpulse: no effect on bodies of the wrong type, wake on request, no accumulation on a
 * sleeping body; SetTransform moves the fixtures' proxies as b2Fixture::Synchronize does).
 * gb_body_edits applies n edits in array order on the device, queued on the handle's stream before
 * the next step (one thread applies them: meant for the sparse changes of a game loop; the whole
 * batch's forces go through gb_set_forces). The edit array may be reused when the call returns. */
#define GB_EDIT_SET_TRANSFORM 0        /* v: position.x, position.y, angle */
#define GB_EDIT_SET_LINEAR_VELOCITY 1  /* v: v.x, v.y */
#define GB_EDIT_SET_ANGULAR_VELOCITY 2 /* v: w */
#define GB_EDIT_SET_AWAKE 3            /* v[0] != 0: awake */
#define GB_EDIT_APPLY_FORCE 4          /* v: force.x, force.y, point.x, point.y (world) */
#define GB_EDIT_APPLY_FORCE_TO_CENTER 5 /* v: force.x, force.y */
#define GB_EDIT_APPLY_TORQUE 6         /* v: torque */
#define GB_EDIT_APPLY_LINEAR_IMPULSE 7 /* v: impulse.x, impulse.y, point.x, point.y (world) */
#define GB_EDIT_APPLY_ANGULAR_IMPULSE 8 /* v: impulse */
#define GB_EDIT_MOUSE_TARGET 9         /* b2MouseJoint::SetTarget (b2MouseJoint.cpp:54): body is the
                                          joint index, v: target.x, target.y (world); wakes body B */
typedef struct gb_body_edit {
    int world;  /* world index in the batch */
    int body;   /* body index (creation order) */
    int op;     /* GB_EDIT_* */
    int wake;   /* the Apply* methods' wake argument */
    float v[4];
} gb_body_edit;
gb_status gb_body_edits(gb_world* world, int n, const gb_body_edit* edits);

/* Whole-batch b2Body::ApplyForceToCenter + ApplyTorque for the next step (Box2D/Dynamics/b2Body.h:
 * 437-468): forces[4] per body of every world in world order then creation order = force.x,
 * force.y, torque, unused. The host array is copied to the device asynchronously on the handle's
 * stream (pinned memory makes it a true async copy); it must stay valid until the next sync. */
gb_status gb_set_forces(gb_world* world, const float* forces);

/* Whole-batch b2Body::GetTransform (Box2D/Dynamics/b2Body.h:180): xf[4] per body of every world in
 * world order then creation order = p.x, p.y, q.s, q.c. Waits for queued steps. */
gb_status gb_get_transforms(gb_world* world, float* xf);

/* Pipelined forms of gb_set_forces and gb_get_transforms for a loop of steps (no reference
 * counterpart; same layouts). gb_set_forces_async copies the host forces into a device staging
 * buffer on an upload stream of the handle, and the handle's stream takes them from there before the
 * next step, so the copy of step k+1's forces overlaps step k. gb_get_transforms_async copies the
 * transforms after the steps queued so far into a staging buffer on the handle's stream and from
 * there to the host on a download stream, overlapping the next step; it does not wait. Two staging
 * buffers per direction are used in turn. The host arrays (pinned memory for true overlap) must stay
 * untouched until gb_world_sync returns, which waits for both transfer streams. */
gb_status gb_set_forces_async(gb_world* world, const float* forces);
gb_status gb_get_transforms_async(gb_world* world, float* xf);

/* The project sin/cos used for every b2Rot (b2Rot::Set, Box2D/Common/b2Math.h:305-312) evaluated on
 * the device for n inputs (host arrays). */
gb_status gb_sincos(const float* x, float* s, float* c, int n);

/* Narrowphase on the device for n shape pairs (b2Collide*, Box2D/Collision/b2Collision.h:170-200):
 * shapes in the gb_create_fixtures encoding, transforms xf[4] = p.x, p.y, q.s, q.c. Output per pair
 * as gb_get_contacts without the first three ints (ints[4]: type, pointCount, id0, id1). */
gb_status gb_collide(int n, const int* type_a, const float* shape_a, const int* n_a, const float* xf_a,
                     const int* type_b, const float* shape_b, const int* n_b, const float* xf_b,
                     int* out_ints, float* out_floats);

/* No counterpart in the reference. gb_collide with no device memory allocation: inputs and outputs
 * are staged in one fixed device buffer defined in the library (static device storage, about
 * 1.7 MB, for at most GB_COLLIDE_NOALLOC_MAX_PAIRS pairs) instead of buffers allocated per call.
 * Arguments, pair rules and output as gb_collide. n > GB_COLLIDE_NOALLOC_MAX_PAIRS returns
 * GB_ERR_CAPACITY before any device work. The buffer is shared by every call on a device: calls
 * whose device work overlaps (for example from several host threads) race on it, so the caller
 * serialises them. The first call on each device resolves the buffer's address
 * (cudaGetSymbolAddress) and should come before any CUDA stream capture. A cudaDeviceReset in the
 * caller's process moves the buffer to a new address in the next context: later calls notice that
 * the cached address is no longer device memory of the current context and resolve it again. */
#define GB_COLLIDE_NOALLOC_MAX_PAIRS 4096
gb_status gb_collide_noalloc(int n, const int* type_a, const float* shape_a, const int* n_a, const float* xf_a,
                             const int* type_b, const float* shape_b, const int* n_b, const float* xf_b,
                             int* out_ints, float* out_floats);

/* ---------------------------------------------------------------- learned warm start
 * No counterpart in the reference. A BF16 MLP 14 -> 64 -> 64 -> 2 (ReLU, FP32 accumulation, tensor
 * cores) that predicts the accumulated normal and tangent impulse of a contact point from 14
 * features of the point at the start of the velocity solve; see gb_world_set_warm_start for the
 * features and how the prediction is used. Parameters are f32 masters, gb_mlp_param_count() of
 * them: W1 [64][16] (inputs 14, 15 zero), b1 [64], W2 [64][64], b2 [64], W3 [8][64] (rows 2..7
 * zero), b3 [8] (2..7 zero), row major [out][in]; features are normalised as (x - mu) / sigma.
 * gb_mlp_forward: y[n][2] for raw features x[n][14] (host arrays). gb_mlp_gradients: loss (mean
 * over rows of the squared error summed over both outputs) and its gradient (param layout) for
 * targets t[n][2], n a multiple of 16, without changing the network. gb_mlp_train: steps of Adam
 * (lr, beta 0.9/0.999) on batches of `batch` rows (a multiple of 16) drawn with a seeded hash from
 * the n rows; losses[steps] (optional) receives each batch's loss. */
gb_status gb_mlp_create(unsigned long long seed, gb_mlp** out);
gb_status gb_mlp_destroy(gb_mlp* mlp);
int gb_mlp_param_count(void);
gb_status gb_mlp_set_params(gb_mlp* mlp, const float* params, const float* mu, const float* sigma);
gb_status gb_mlp_get_params(gb_mlp* mlp, float* params, float* mu, float* sigma);
gb_status gb_mlp_forward(gb_mlp* mlp, const float* x, int n, float* y);
gb_status gb_mlp_gradients(gb_mlp* mlp, const float* x, const float* t, int n, float* grad, float* loss);
gb_status gb_mlp_train(gb_mlp* mlp, const float* x, const float* t, int n, int steps, int batch, float lr,
                       unsigned long long seed, float* losses);

/* Warm start of the following steps (no counterpart in the reference). GB_WARM_REFERENCE (default)
 * is b2ContactSolver's: each point starts from its previous impulses scaled by dtRatio
 * (Box2D/Dynamics/Contacts/b2ContactSolver.cpp:100-110, 254-292). GB_WARM_LEARNED evaluates the
 * network for every island contact point after the constraints are initialised, from 14 features:
 * world normal (2); relative normal and tangent velocity at the point; its separation; inverse mass
 * and inertia of both bodies (4); the reference warm-start normal and tangent impulses divided by
 * the point's normal and tangent effective mass; the effective inverse normal mass; the friction
 * coefficient; 1 for a two-point manifold. The outputs, multiplied by the normal and tangent
 * effective mass, are corrections added to the reference warm-start impulses (the normal result
 * clamped at 0, the tangent one to the friction cone), applied at the points the reference starts
 * cold (no normal impulse carried over); the network is trained on such logged points, on the final
 * impulses minus the reference warm start (t - x[9..10] in the log's units). GB_WARM_LEARNED_ALL
 * applies the corrections at every point (a network trained on all logged points).
 * Each world then warm-starts its velocities both ways and keeps the one whose velocity residual is
 * smaller, island by island (islands share no dynamic body), so an island falls back to the reference
 * warm start whenever the prediction is worse. The network must outlive its use by the world. */
#define GB_WARM_REFERENCE 0
#define GB_WARM_LEARNED 1
#define GB_WARM_LEARNED_ALL 2
gb_status gb_world_set_warm_start(gb_world* world, gb_mlp* mlp, int mode);
/* Per world of the last step (arrays of n_worlds, each may be NULL): islands that kept the learned
 * warm start, and the contact-iterations of the velocity solve (each island's iterations times its
 * contacts, summed): divided by the solved contacts (gb_world_totals), the mean iterations a contact
 * went through, e.g. to reach a residual tolerance. */
gb_status gb_world_warm_stats(gb_world* world, int* learned_islands, int* vel_iters_sum);

/* Contact-point log for training the network (plain solver only): capacity > 0 allocates a device
 * log of that many points and starts recording, 0 stops and frees it. Every step appends, for each
 * island contact point of every world, its 14 features at the start of the velocity solve (x) and
 * the normal and tangent impulses the velocity iterations end with divided by the effective masses
 * (t, the network's targets). gb_world_read_contact_log copies up to cap points to the host, sets *n,
 * empties the log and returns GB_ERR_CAPACITY when points were dropped for lack of room. */
gb_status gb_world_set_contact_log(gb_world* world, int capacity);
gb_status gb_world_read_contact_log(gb_world* world, float* x, float* t, int cap, int* n);

/* Library version string. */
const char* gb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BOX2D_GB300_H */
