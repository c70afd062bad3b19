// Oracle (test infrastructure only): world, bodies, fixtures, contacts, joints, island and contact
// solver declarations for the CPU restatement of Box2D 2.3.2 b2World::Step.
#pragma once
#include "tree.h"

namespace b2o {

enum BodyType { kStatic = 0, kKinematic = 1, kDynamic = 2 };
// b2Body flags (Dynamics/b2Body.h:409-418)
enum : uint32_t { kBIsland = 0x1, kBAwake = 0x2, kBAutoSleep = 0x4, kBBullet = 0x8, kBFixedRot = 0x10, kBActive = 0x20, kBToi = 0x40 };
// b2Contact flags (Dynamics/Contacts/b2Contact.h:158-177)
enum : uint32_t { kCIsland = 0x1, kCTouching = 0x2, kCEnabled = 0x4, kCFilter = 0x8, kCBulletHit = 0x10, kCToi = 0x20 };

struct Body {
    int type = kStatic;
    uint32_t flags = 0;
    int islandIndex = 0;
    Xf xf{};
    Sweep sweep{};
    Vec2 v{0, 0};
    float w = 0;
    Vec2 force{0, 0};
    float torque = 0;
    float mass = 0, invMass = 0, I = 0, invI = 0;
    float linearDamping = 0, angularDamping = 0, gravityScale = 1, sleepTime = 0;
    int prev = kNull, next = kNull;
    int fixtureList = kNull;
    int contactList = kNull; // edge id: contact * 2 + side
    int jointList = kNull;   // edge id: joint * 2 + side
    bool alive = true;       // false once destroyed (its dump is zeros)
    bool IsAwake() const { return (flags & kBAwake) != 0; }
};

struct Fixture {
    int body = kNull, next = kNull;
    Shape shape;
    float density = 0, friction = 0.2f, restitution = 0;
    uint16_t category = 1, mask = 0xFFFF;
    int16_t group = 0;
    bool sensor = false;
    int proxyId = kNull;
    int proxyCount = 0;
    AABB aabb{};
};

struct Contact {
    uint32_t flags = 0;
    int fA = kNull, fB = kNull, iA = 0, iB = 0;
    Manifold m{};
    int toiCount = 0;
    float toi = 1.0f;
    float friction = 0, restitution = 0, tangentSpeed = 0;
    int prev = kNull, next = kNull;
    int ePrev[2] = {kNull, kNull}, eNext[2] = {kNull, kNull};
    bool alive = false;
};

// joint types (b2JointType, Dynamics/Joints/b2Joint.h:28-42, those restated here)
enum JointType { kRevoluteJoint = 0, kDistanceJoint = 1, kWeldJoint = 2, kPrismaticJoint = 3, kWheelJoint = 4,
                 kRopeJoint = 5, kFrictionJoint = 6, kMotorJoint = 7, kMouseJoint = 8, kPulleyJoint = 9, kGearJoint = 10 };

struct Joint {
    int type = kRevoluteJoint;
    int bodyA = kNull, bodyB = kNull;
    bool collideConnected = false, islandFlag = false;
    int prev = kNull, next = kNull;
    int ePrev[2] = {kNull, kNull}, eNext[2] = {kNull, kNull};
    // revolute joint (Dynamics/Joints/b2RevoluteJoint.h)
    Vec2 localAnchorA{0, 0}, localAnchorB{0, 0};
    float referenceAngle = 0, lowerAngle = 0, upperAngle = 0, maxMotorTorque = 0, motorSpeed = 0;
    bool enableLimit = false, enableMotor = false;
    float impulse[3] = {0, 0, 0};
    float motorImpulse = 0;
    int limitState = 0; // 0 inactive, 1 lower, 2 upper, 3 equal
    int indexA = 0, indexB = 0;
    Vec2 rA{0, 0}, rB{0, 0}, localCenterA{0, 0}, localCenterB{0, 0};
    float invMassA = 0, invMassB = 0, invIA = 0, invIB = 0;
    float mass[9] = {0};     // b2Mat33 columns ex, ey, ez
    float motorMass = 0;
    // distance joint (b2DistanceJoint.h): length, spring; weld joint (b2WeldJoint.h): spring (the
    // weld's reference angle is referenceAngle, its impulse impulse[0..2], its mass mass[])
    float length = 0, frequencyHz = 0, dampingRatio = 0;
    float gamma = 0, bias = 0;
    Vec2 u{0, 0};            // distance: unit axis of the step (its effective mass in motorMass); prismatic: axis
    // prismatic joint (b2PrismaticJoint.h): translation limits in lowerAngle/upperAngle, maximum motor
    // force in maxMotorTorque, the 3x3 K in mass[]
    Vec2 localXAxisA{0, 0}, localYAxisA{0, 0}, perp{0, 0};
    float s1 = 0, s2 = 0, a1 = 0, a2 = 0;
    // wheel joint (b2WheelJoint.h): point-on-line mass in mass[0], motor torque and speed in
    // maxMotorTorque, motorSpeed
    Vec2 ax{0, 0}, ay{0, 0};
    float sAx = 0, sBx = 0, sAy = 0, sBy = 0, springMass = 0, springImpulse = 0;
    // rope joint (b2RopeJoint.h): impulse in impulse[0], mass in motorMass, state in limitState
    float maxLength = 0, ropeLength = 0;
    // friction and motor joints: linear impulse impulse[0..1], angular impulse[2], 2x2 linear mass
    // mass[0..3] (columns ex, ey), angular mass motorMass
    float maxForce = 0, maxTorque = 0;
    Vec2 linearOffset{0, 0}, linearError{0, 0};
    float angularOffset = 0, angularError = 0, correctionFactor = 0;
    // mouse joint (b2MouseJoint.h): soft point-to-target spring on body B; impulse[0..1], the 2x2 mass
    // in mass[0..3], gamma as the distance joint's
    Vec2 target{0, 0}, mouseC{0, 0};
    float beta = 0;
    // pulley joint (b2PulleyJoint.h): impulse in impulse[0], effective mass in motorMass
    Vec2 groundAnchorA{0, 0}, groundAnchorB{0, 0}, uA{0, 0}, uB{0, 0};
    float lengthA = 0, lengthB = 0, ratio = 1, pulleyConstant = 0;
    // gear joint (b2GearJoint.h): joint 1 couples bodies C and A, joint 2 D and B (bodyA/bodyB here);
    // A's reference angle in referenceAngle; impulse in impulse[0], mass in motorMass
    int bodyC = kNull, bodyD = kNull, typeA = 0, typeB = 0, indexC = 0, indexD = 0;
    Vec2 localAnchorC{0, 0}, localAnchorD{0, 0}, localAxisC{0, 0}, localAxisD{0, 0};
    Vec2 lcC{0, 0}, lcD{0, 0};
    float referenceAngleB = 0, gearConstant = 0, invMassC = 0, invMassD = 0, invIC = 0, invID = 0;
    Vec2 JvAC{0, 0}, JvBD{0, 0};
    float JwA = 0, JwB = 0, JwC = 0, JwD = 0;
};

struct Position { Vec2 c; float a; };
struct Velocity { Vec2 v; float w; };
struct StepInfo { float dt, inv_dt, dtRatio; int velocityIterations, positionIterations; bool warmStarting; };

struct Event { int kind, fA, fB; float n0, n1, t0, t1; }; // kind: 0 begin, 1 end, 2 presolve, 3 postsolve

struct World {
    Vec2 gravity{0, -10};
    std::vector<Body> bodies;
    std::vector<Fixture> fixtures;
    std::vector<Contact> contacts;
    std::vector<int> freeContacts;
    std::vector<Joint> joints;
    int bodyList = kNull, contactList = kNull, jointList = kNull;
    int bodyCount = 0, contactCount = 0, jointCount = 0;
    uint32_t wflags = 0x4; // e_clearForces
    bool allowSleep = true, warmStarting = true, continuous = true, subStepping = false, stepComplete = true;
    float inv_dt0 = 0;
    BroadPhase bp;
    bool recordEvents = false;
    std::vector<Event> events;
    std::vector<Pair> stepPairs; // every UpdatePairs list of the last step, separated by {-1,-1}
    // island scratch
    std::vector<int> iBodies, iContacts, iJoints, stack;
    std::vector<Position> positions;
    std::vector<Velocity> velocities;

    // A PreSolve listener's rule, per fixture: bit 0 ghost, 1 ice, 2 bouncy; a contact between two
    // fixtures sharing a bit is disabled (ghost), gets friction 0 (ice) or restitution 0.9 (bouncy).
    std::vector<int> preSolveRule;
    // A test b2ContactFilter (filterModulus > 0): fixtures below filterStatic use the default filter;
    // any other pair collides unless (fixtureA + fixtureB) % filterModulus == 0.
    int filterModulus = 0, filterStatic = 0;
    bool DefaultFilter(int fA, int fB) const;
    bool FilterShouldCollide(int fA, int fB) const;
    // destruction listener calls of the last Destroy* call: {0 joint / 1 fixture, index}
    std::vector<std::pair<int, int>> goodbyes;
    void DestroyBody(int b);
    void DestroyJoint(int j);
    void DestroyFixture(int f);
    int CreateBody(int type, const float* f, int flags);
    int CreateFixture(int body, const Shape& shape, float density, float friction, float restitution,
                      int category, int mask, int group, bool sensor);
    int CreateRevolute(int a, int b, const float* f, int flags);
    int CreateJoint(int type, int a, int b, const float* f, int flags);
    int LinkJoint(Joint& j, int a, int b);
    void ResetMassData(int b);
    void SetAwake(int b, bool flag);
    bool ShouldCollide(int bodyB, int bodyA) const;
    void SynchronizeFixtures(int b);
    void SynchronizeFixturesFrom(int b, const Xf& xf1, const Xf& xf2);
    void ApplyEdit(int op, int b, int wake, const float* v);
    // b2Body property changes between steps (the C-ABI's GB_BODY_* prop codes)
    void SetBodyProperty(int b, int prop, const float* v);
    void SetFixtureProperty(int f, int prop, const float* v);
    void ShiftOrigin(Vec2 origin);
    int SetJointProperty(int j, int prop, const float* v);
    void SynchronizeTransform(int b);
    void Advance(int b, float alpha);

    void FindNewContacts();
    void AddPair(int proxyA, int proxyB);
    void Destroy(int c);
    void Collide();
    void Update(int c);
    void Evaluate(int c, Manifold* m);
    void Solve(const StepInfo& step);
    void SolveTOI(const StepInfo& step);
    void IslandSolve(const StepInfo& step);
    void IslandSolveTOI(const StepInfo& sub, int toiA, int toiB);
    void Step(float dt, int vi, int pi);

    int EdgeOther(int e) const;
    int JointEdgeOther(int e) const;
    int Link(int c);
};

} // namespace b2o
