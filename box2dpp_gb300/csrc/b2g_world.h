// Device-resident world state for the GB300 Box2D step.
//
// A batch holds W independent worlds; one world is a batch of one. Every per-body, per-fixture,
// per-proxy and per-contact column lives in HBM for the whole run as a structure of arrays of 16-byte
// vectors (float4/int4), indexed world-locally through the world's base offsets. The host writes it
// at upload and reads it back on demand; a step never leaves the device.
#pragma once

#include <cstdint>
#include <vector_types.h>

#include "b2g_core.h"
#include "b2g_mlp.cuh"

namespace b2g {

constexpr int kNullIdx = -1;

// b2Body flags (Dynamics/b2Body.h:409-418)
enum : int { kBIsland = 0x1, kBAwake = 0x2, kBAutoSleep = 0x4, kBBullet = 0x8, kBFixedRot = 0x10, kBActive = 0x20 };
// b2Contact flags (Dynamics/Contacts/b2Contact.h:158-177)
enum : int { kCIsland = 0x1, kCTouching = 0x2, kCEnabled = 0x4, kCFilter = 0x8, kCToi = 0x20 };
enum BodyType { kStatic = 0, kKinematic = 1, kDynamic = 2 };

// Status words (the C-ABI's gb_status values are the host mirror of these bits).
enum : int { kErrCapacity = 1, kErrTimeout = 2, kErrInvalid = 4 };

// Per-world sizes and base offsets into the batch columns (immutable during a step).
struct WorldDesc {
    int bodyBase, bodyCount;
    int fixBase, fixCount;
    int proxyBase, proxyCap;
    int contactBase, contactCap;
    int jointBase, jointCount;
    int pairBase, pairCap;
    // island rows: a static body is a row of every island it touches, so rows can exceed bodies
    int rowBase, rowCap;
    // island-table region (bytes) for the DFS when its table does not fit in shared memory
    long long islTabBase;
    int islTabBytes;
};

constexpr int kProfileSlots = 24;
// Rows per chunk of the flat pre-passes (NarrowphaseKernel, ToiKernel): one CTA of kRowChunk threads
// per chunk of one world's contact (or body) rows; the chunks are listed in schedule order, so a
// class of the launch plan launches exactly its own worlds' chunks.
constexpr int kRowChunk = 128;

// Per-world mutable scalars.
struct WorldState {
    float gx, gy;
    float inv_dt0;
    int bodyList;       // head of the body list (newest body first)
    int jointList;
    int contactCount;   // live contacts == length of the contact order list
    int freeContact;    // head of the contact-slot free list
    int newFixture;     // b2World::e_newFixture
    int stepComplete;
    int allowSleep, warmStarting, continuous, subStepping;
    int clearForces;    // b2World's e_clearForces: forces and torques cleared at the end of each step
    int error;          // kErr* bits
    int toiEvents;      // TOI sub-steps taken in the last step (diagnostic)
    int islands;        // islands solved in the last step (diagnostic)
    int solvedBodies;   // non-static island rows solved in the last step
    int solvedContacts; // island contacts solved in the last step
    int pairsFound;     // broadphase pairs produced in the last step (all UpdatePairs calls)
    int colours;        // constraint colours used by the coloured solver in the last step
    int velIters;       // velocity iterations run in the last step (fewer than asked when a tolerance is met)
    float residual;     // velocity residual (m/s) after the last step's velocity iterations, when measured
    int warmLearned;    // islands of the last step that kept the learned warm start (its residual was smaller)
    int velItersSum;    // velocity iterations of the last step x island contacts, summed over islands
    float maxPenetration; // deepest contact penetration (m) before the last step's position correction
    int eventCount;     // listener records of the last step in the world's event log
    int eventsDropped;  // 1 when the log ran out of room
    int staged;         // 1 while this step's manifolds wait in the stage (NarrowphaseKernel -> collide)
    int toiPrepared;    // 1 while this step's first time-of-impact pass is done (ToiKernel -> solveTOI)
    // the uniform grid of the step's pair finding, kept for the continuous phase's events (cells as
    // linked lists that an event's moved proxies relink): valid while gridValid is 1
    int gridValid, gridNx, gridNy, gridLive;
    // the contact list (newest first) is order[orderStart, orderStart + contactCount) of the world's
    // 2 x contactCap order rows: new contacts are prepended in front of it without moving the rest
    int orderStart;
    float gridOx, gridOy, gridInvH, gridW, gridWLarge;
    int treeLogCount;   // records written to the world's tree log since the host last read it
    // SM clock cycles of the last step per phase: 0 new-fixture pairs, 1 collide, 2 island DFS,
    // 3 island solve, 4 fixture sync, 5 pairs after solve, 6 TOI, 7 whole step; then the island solve
    // split: 8 integrate + constraint init, 9 warm start + velocity sweeps, 10 impulses + position
    // integration, 11 position sweeps, 12 write-back, 13 sleep; 14 pair finding and sorting, 15 contact
    // creation (both summed over every UpdatePairs call of the step); the TOI split (summed over its
    // events): 16 contact classification and time of impact, 17 earliest-event selection, 18 event
    // mini-island build, 19 mini-island solve, 20 fixture sync and contact invalidation, 21 pair
    // finding after events; 22, 23 unused (the flat pre-pass kernels are not counted per world)
    unsigned long long cyc[kProfileSlots];
};

// Joint types (b2JointType, Dynamics/Joints/b2Joint.h:28-42, those built here).
enum : int { kJointRevolute = 0, kJointDistance = 1, kJointWeld = 2, kJointPrismatic = 3, kJointWheel = 4,
             kJointRope = 5, kJointFriction = 6, kJointMotor = 7, kJointMouse = 8, kJointPulley = 9, kJointGear = 10, kJointTypes };

// A joint (Dynamics/Joints/b2RevoluteJoint.h, b2DistanceJoint.h, b2WeldJoint.h), stored whole: joints
// are few. Fields a type does not use stay zero; the distance joint keeps its scalar impulse in
// impulse[0] and its effective mass in motorMass, the weld joint its 3x3 effective mass in mass[].
struct Joint {
    int type;
    int bodyA, bodyB;
    int collideConnected, islandFlag;
    int prev, next;
    int ePrev[2], eNext[2];
    Vec2 localAnchorA, localAnchorB;
    float referenceAngle, lowerAngle, upperAngle, maxMotorTorque, motorSpeed;
    int enableLimit, enableMotor;
    float impulse[3];
    float motorImpulse;
    int limitState;
    int indexA, indexB;
    Vec2 rA, rB, localCenterA, localCenterB;
    float invMassA, invMassB, invIA, invIB;
    float mass[9];
    float motorMass;
    float length, frequencyHz, dampingRatio;  // distance: length; distance, weld: spring
    float gamma, bias;                        // soft constraint terms of the step
    Vec2 u;                                   // distance: unit axis of the step; prismatic: axis
    Vec2 localXAxisA, localYAxisA;            // prismatic: unit axis in body A and its normal
    Vec2 perp;                                // prismatic: normal of the axis, this step
    float s1, s2, a1, a2;                     // prismatic: lever arms of the step
    // wheel (b2WheelJoint.h): the axis in localXAxisA/localYAxisA, this step's axes and lever arms,
    // spring and motor state (the motor's maximum torque and speed in maxMotorTorque, motorSpeed)
    Vec2 ax, ay;
    float sAx, sBx, sAy, sBy;
    float springMass, springImpulse;
    // rope (b2RopeJoint.h): maximum length, this step's length; its impulse in impulse[0], mass in
    // motorMass, state in limitState
    float maxLength, ropeLength;
    // friction and motor (b2FrictionJoint.h, b2MotorJoint.h): linear impulse in impulse[0..1], angular
    // in impulse[2], the 2x2 linear mass in mass[0..3] (b2Mat22 columns ex, ey), angular mass in
    // motorMass
    float maxForce, maxTorque;
    Vec2 linearOffset, linearError;           // motor
    float angularOffset, angularError, correctionFactor;
    // mouse (b2MouseJoint.h): target point (world), this step's position error; maxForce, the spring
    // in frequencyHz / dampingRatio, the 2x2 mass in mass[0..3], the impulse in impulse[0..1]
    Vec2 target, mouseC;
    float beta;
    // pulley (b2PulleyJoint.h): ground anchors, lengths, ratio, constant; this step's unit vectors
    // uA, uB; the impulse in impulse[0], mass in motorMass
    Vec2 groundAnchorA, groundAnchorB, uA, uB;
    float lengthA, lengthB, ratio, pulleyConstant;
    // gear (b2GearJoint.h): couples a revolute or prismatic joint 1 (bodies C, A) with joint 2 (D, B);
    // bodyA/bodyB are the joints' bodies B, localAnchorA/B and referenceAngle (A's) theirs, the axes
    // zero for a revolute joint; ratio as the pulley's; this step's Jacobian, the island rows and mass
    // data of C and D; the impulse in impulse[0], mass in motorMass
    int bodyC, bodyD, indexC, indexD, gearTypeA, gearTypeB;
    Vec2 localAnchorC, localAnchorD, localAxisC, localAxisD, localCenterC, localCenterD;
    float referenceAngleB, gearConstant, invMassC, invMassD, invIC, invID;
    Vec2 JvAC, JvBD;
    float JwA, JwB, JwC, JwD;
};

// Island solver records: the fields of b2ContactVelocityConstraint and b2ContactPositionConstraint
// (Dynamics/Contacts/b2ContactSolver.h:35-56, b2ContactSolver.cpp:34-47) regrouped into 16-byte
// vectors so a record loads with a few 128-bit loads. The accumulated impulses, the only part the
// velocity sweeps write, live in a separate float4 per contact {normal0, tangent0, normal1, tangent1}.
struct __align__(16) VelConstraint {
    float4 nf;   // normal.x, normal.y, friction, tangentSpeed
    float4 m;    // invMassA, invIA, invMassB, invIB
    int4 idx;    // indexA (body row), indexB, pointCount, contact slot
    float4 K;    // block matrix ex.x, ex.y, ey.x, ey.y
    float4 NM;   // its inverse (normalMass)
    float4 r0;   // point 0: rA.x, rA.y, rB.x, rB.y
    float4 c0;   // point 0: normalMass, tangentMass, velocityBias, restitution
    float4 r1;   // point 1
    float4 c1;
};
struct __align__(16) PosConstraint {
    float4 lp;   // localPoints[0].xy, localPoints[1].xy
    float4 ln;   // localNormal.xy, localPoint.xy
    int4 idx;    // indexA, indexB, pointCount, manifold type
    float4 m;    // invMassA, invIA, invMassB, invIB
    float4 lc;   // localCenterA.xy, localCenterB.xy
    float4 rad;  // radiusA, radiusB, 0, 0
};
struct TOITask { int contact; int kind; float alpha0; Sweep sa, sb; };

// A contact's manifold as b2Contact::Update would leave it (evaluated, impulses matched by id) but
// not yet committed, written by NarrowphaseKernel before the step and read by the collide phase.
// It lives in the contact's VelConstraint slot, which is free until the island solve. tag is 1 when
// the record belongs to this step; 0 when the contact was left to the collide phase.
struct __align__(16) ManifoldStage {
    int4 h;      // type, pointCount, id0, id1
    float4 v;    // localNormal.xy, localPoint.xy
    float4 p0;   // point 0: localPoint.xy, normalImpulse, tangentImpulse
    float4 p1;   // point 1
    int tag;
};
static_assert(sizeof(ManifoldStage) <= sizeof(VelConstraint), "the stage reuses a VelConstraint slot");

// All columns of a batch. Per world, column x of world w starts at x + desc[w].<kind>Base.
struct Batch {
    int worlds;
    int bodyRows, contactRows;  // lengths of the body and contact columns (all worlds, padding included)
    WorldDesc* desc;
    WorldState* state;
    int* bWorld;   // body-column row -> its world (the flat pre-pass kernels' map)
    int* cWorld;   // contact-column row -> its world
    // bodies
    float4* xf;    // p.x, p.y, q.s, q.c
    float4* sw;    // c.x, c.y, a, alpha0
    float4* sw0;   // c0.x, c0.y, a0, sleepTime
    float4* vel;   // v.x, v.y, w, 0
    float4* frc;   // force.x, force.y, torque, 0
    float4* mas;   // invMass, invI, localCenter.x, localCenter.y
    float4* prop;  // linearDamping, angularDamping, gravityScale, mass
    int4* bi;      // type, flags, fixtureList, contactList (edge id = 2*slot + side)
    int4* bj;      // jointList (edge id = 2*joint + side), bodyNext, islandIndex, wake scratch
    // fixtures
    int4* fi;      // body, next, proxyId, isSensor
    float4* fm;    // friction, restitution, density, radius
    int4* ff;      // categoryBits, maskBits, groupIndex, 0
    float4* faabb; // swept AABB last synchronised (b2FixtureProxy::aabb)
    Shape* shape;
    // proxies (indexed by proxy id, the reference's tree node id)
    float4* fat;   // fat AABB
    int* pfix;     // fixture of the proxy, -1 when free
    int* moved;    // in the move buffer
    // contacts (slots)
    int4* ci;      // flags, fixtureA, fixtureB, toiCount
    int4* ce;      // ePrev[0], eNext[0], ePrev[1], eNext[1]  (edge 0 on bodyA's list, 1 on bodyB's)
    float4* cp;    // friction, restitution, tangentSpeed, toi
    int4* mh;      // manifold type, pointCount, id0, id1
    float4* mv;    // localNormal.xy, localPoint.xy
    float4* mp0;   // point 0: localPoint.xy, normalImpulse, tangentImpulse
    float4* mp1;   // point 1
    int* order;    // live contacts in world-list order (newest first), length state.contactCount
    int* cnext;    // free-list link of a free slot
    // joints
    Joint* joint;
    // scratch (per world, same bases)
    int* sBody;      // row-sized: island bodies
    int* sStack;     // body-sized: DFS stack / wake positions
    int* sWake;
    float4* sPos;    // row-sized island positions c.x, c.y, a
    float4* sVel;    // row-sized island velocities v.x, v.y, w
    int* sContact;   // contact-sized: island contact list / collide status / pair keep flags
    int* sStatus;
    VelConstraint* vc;
    PosConstraint* pc;
    float4* vimp;    // contact-sized impulses of the island contacts (when not staged in shared memory)
    float4* vimpL;   // contact-sized learned warm-start impulses
    float2* vsep;    // contact-sized separations of the points at the start of the velocity solve
    float4* sVelL;   // row-sized velocities under the learned warm start
    TOITask* toi;
    int4* islands;   // body-sized: {bodyStart, bodyCount, contactStart, contactCount}
    int2* islandJ;   // {jointStart, jointCount}
    int* sJoint;     // joint-sized
    int* sleepOut;   // per island: 1 when the island fell asleep
    int* cColour;    // contact-sized: colour of each island contact (coloured solver)
    int* evType;     // contact-sized: listener calls of each list position in the collide phase
    int4* evLog;     // 4 x contact-sized records of 2 int4, or nullptr when events are off: the step's
                     // listener calls {kind 0 begin, 1 end, 2 pre-solve, 3 post-solve, fixtureA,
                     // fixtureB, impulse points} {normal impulse 0, 1, tangent impulse 0, 1}
    int* colourList; // contact-sized: island contacts grouped by colour
    unsigned long long* rowMask; // row-sized: colours used at each island body row
    unsigned long long* pairs; // pair-sized sort keys (proxyA << 32 | proxyB)
    int* pairKeep;
    int4* pairInfo;  // pair-sized: a new contact's fixtures and bodies, worked out before creation
    int* movedList;  // proxy-sized
    int* liveProxies; // proxy-sized: pair finding's list of live proxies when it is not in shared memory
    int* gridIds;     // proxy-sized: the live proxies of the kept grid
    int* gridNext;    // proxy-sized: next proxy in the same cell list (-1 at the end)
    int* gridPrev;    // proxy-sized: previous proxy in the same cell list (-1 at the head)
    int* gridCellOf;  // proxy-sized: the cell list holding the proxy (nx * ny: the large proxies' list)
    int* gridHead;    // pair-sized: first proxy of each cell list (nx * ny + 1 lists)
    unsigned char* islTab; // island-DFS tables of the worlds whose table does not fit in shared memory
    // A user contact filter (b2World::SetContactFilter): verdicts of b2ContactFilter::ShouldCollide per
    // (world, fixtureA, fixtureB) in an open-addressing table (filterCap slots, a power of two; key
    // ~0 empty; value 1 collide, 0 not, 2 not known yet), and the pairs met without a verdict:
    // filterMiss[0] their count, then (world, fixtureA, fixtureB) triples, at most filterMissCap.
    // filterKeys == nullptr: the default filter (category, mask, group) runs on the device.
    unsigned long long* filterKeys;
    int* filterVals;
    int filterCap;
    int* filterMiss;
    int filterMissCap;
    // The tree log (b2World::GetTreeHeight and the other tree diagnostics), or nullptr when no world
    // of the batch keeps its tree: every fat box the device gives a proxy (b2DynamicTree::MoveProxy
    // re-inserting the leaf), world w's records at kTreeLogPerProxy * proxyBase + kTreeLogExtra * w,
    // kTreeLogPerProxy * proxyCap + kTreeLogExtra of them. treeLogId = proxy << 2 | kind (TreeLogKind).
    int* treeLogId;
    float4* treeLogFat;
};

// Records of the tree log per proxy slot and per world.
constexpr int kTreeLogPerProxy = 8;
constexpr int kTreeLogExtra = 256;
// Kinds of tree-log records: kTreeOrdered re-insertions happen in log order (body edits between steps,
// the continuous phase's events); the kTreeDiscrete ones are the discrete phase's fixture
// synchronisation, written by many threads at once, whose order is the world's body list, then each
// body's fixture list (b2World::Solve, Dynamics/b2World.cpp:494-514); kTreeStepMark opens a step's
// discrete records.
enum TreeLogKind : int { kTreeOrdered = 0, kTreeDiscrete = 1, kTreeStepMark = 2 };

// Key and first probe of a verdict in the contact-filter table (fixtures below 2^20 per world).
B2G_HD unsigned long long FilterKey(int w, int fA, int fB)
{
    return ((unsigned long long)(unsigned)w << 40) | ((unsigned long long)(unsigned)fA << 20) | (unsigned)fB;
}
B2G_HD unsigned FilterSlot(unsigned long long key, int cap)
{
    unsigned long long h = key * 0x9E3779B97F4A7C15ull;
    return (unsigned)(h >> 32) & (unsigned)(cap - 1);
}

// A change to a contact between the halves of a split step (the device copy of gb_contact_edit):
// contact = position in the world's contact list; flags bit 0 enabled, 1 friction, 2 restitution,
// 3 tangent speed.
struct ContactEdit {
    int world, contact, flags, enabled;
    float friction, restitution, tangentSpeed, pad;
};

// A b2Body state change between steps (the device copy of the C-ABI's gb_body_edit, same layout).
enum : int { kEditSetTransform = 0, kEditSetLinearVelocity, kEditSetAngularVelocity, kEditSetAwake, kEditApplyForce,
             kEditApplyForceToCenter, kEditApplyTorque, kEditApplyLinearImpulse, kEditApplyAngularImpulse,
             kEditMouseTarget, kEditOps };
struct BodyEdit {
    int world, body, op, wake;
    float v[4];
};

// Island solver variants. kSolverPlain is the reference's per-island sequential Gauss-Seidel order
// (bit-exact with the reference). kSolverColoured solves the same constraints colour by colour: the
// constraints of one colour share no dynamic body and are solved in parallel across the CTA.
enum : int { kSolverPlain = 0, kSolverColoured = 1 };
enum : int { kWarmReference = 0, kWarmLearned = 1, kWarmLearnedAll = 2 };
// b2ContactListener calls (Dynamics/b2WorldCallbacks.h:84-130) as event log kinds
enum : int { kEvBegin = 0, kEvEnd = 1, kEvPreSolve = 2, kEvPostSolve = 3 };
// Colours 0..62 are solved in parallel; colour 63 collects the constraints for which no colour was
// free and is solved by one thread in island order.
constexpr int kColours = 64;
constexpr int kSerialColour = kColours - 1;

// Shared-memory shape of one step launch: island rows and contacts staged per CTA.
struct LaunchShape {
    int smemRows, smemContacts;
};

struct StepParams {
    float dt;
    int velocityIterations, positionIterations;
    int maxToiEvents;   // bound on TOI sub-steps per world per step (error bit on overflow)
    int solver;         // kSolverPlain or kSolverColoured
    float tolerance;    // > 0: stop the velocity iterations once the velocity residual is <= tolerance
    int measureResidual;// 1: record the velocity residual after the velocity iterations
    int recordEvents;   // 1: record the listener calls of the step in the event log
    int phase;          // 0 the whole step; 1 up to the collide phase; 2 the rest (a step split for a
                        // PreSolve that changes contacts)
    int warmMode;       // kWarmReference, kWarmLearned or kWarmLearnedAll (the network below, reference as fallback)
    MlpView mlp;
    // contact-point log (plain solver): features at the start of the velocity solve, then the
    // scaled impulses the velocity iterations end with; logX == nullptr disables it
    float* logX;        // [logCap][14]
    float* logT;        // [logCap][2]
    int* logCount;
    int logCap;
};

} // namespace b2g
