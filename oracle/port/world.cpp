// Oracle (test infrastructure only): the CPU restatement of Box2D 2.3.2 b2World::Step with its
// contact manager, island builder, island solver, contact solver, continuous (TOI) pass and revolute
// joint. Paths are relative to the reference tree's Regression/box2d-ref/Box2DRef/.
#include "world.h"

#include <cstring>

namespace b2o {

// ---------------------------------------------------------------- bodies, fixtures, joints
// b2World::CreateBody (Dynamics/b2World.cpp:115-140) + b2Body::b2Body (Dynamics/b2Body.cpp:27-107)
int World::CreateBody(int type, const float* f, int fl)
{
    Body b;
    b.flags = 0;
    if (fl & 8) b.flags |= kBBullet;
    if (fl & 4) b.flags |= kBFixedRot;
    if (fl & 1) b.flags |= kBAutoSleep;
    if (fl & 2) b.flags |= kBAwake;
    if (fl & 16) b.flags |= kBActive;
    b.xf.p = V(f[0], f[1]);
    b.xf.q = RotOf(f[2]);
    b.sweep.localCenter = V(0.0f, 0.0f);
    b.sweep.c0 = b.xf.p;
    b.sweep.c = b.xf.p;
    b.sweep.a0 = f[2];
    b.sweep.a = f[2];
    b.sweep.alpha0 = 0.0f;
    b.v = V(f[3], f[4]);
    b.w = f[5];
    b.linearDamping = f[6];
    b.angularDamping = f[7];
    b.gravityScale = f[8];
    b.type = type;
    if (type == kDynamic) { b.mass = 1.0f; b.invMass = 1.0f; }
    int id = (int)bodies.size();
    b.prev = kNull;
    b.next = bodyList;
    bodies.push_back(b);
    if (bodyList != kNull) bodies[bodyList].prev = id;
    bodyList = id;
    ++bodyCount;
    return id;
}

// b2Body::ResetMassData (Dynamics/b2Body.cpp:283-352)
void World::ResetMassData(int bi)
{
    Body& b = bodies[bi];
    b.mass = 0.0f; b.invMass = 0.0f; b.I = 0.0f; b.invI = 0.0f;
    b.sweep.localCenter = V(0.0f, 0.0f);
    if (b.type == kStatic || b.type == kKinematic) {
        b.sweep.c0 = b.xf.p;
        b.sweep.c = b.xf.p;
        b.sweep.a0 = b.sweep.a;
        return;
    }
    Vec2 localCenter = V(0.0f, 0.0f);
    for (int f = b.fixtureList; f != kNull; f = fixtures[f].next) {
        if (fixtures[f].density == 0.0f) continue;
        MassData md;
        ComputeMass(fixtures[f].shape, fixtures[f].density, &md);
        b.mass += md.mass;
        localCenter = localCenter + md.mass * md.center;
        b.I += md.I;
    }
    if (b.mass > 0.0f) {
        b.invMass = 1.0f / b.mass;
        localCenter.x *= b.invMass;
        localCenter.y *= b.invMass;
    } else {
        b.mass = 1.0f;
        b.invMass = 1.0f;
    }
    if (b.I > 0.0f && (b.flags & kBFixedRot) == 0) {
        b.I -= b.mass * Dot(localCenter, localCenter);
        b.invI = 1.0f / b.I;
    } else {
        b.I = 0.0f;
        b.invI = 0.0f;
    }
    Vec2 oldCenter = b.sweep.c;
    b.sweep.localCenter = localCenter;
    b.sweep.c = Mul(b.xf, b.sweep.localCenter);
    b.sweep.c0 = b.sweep.c;
    b.v = b.v + Cross(b.w, b.sweep.c - oldCenter);
}

// b2Body::CreateFixture (Dynamics/b2Body.cpp:165-201) + b2Fixture::CreateProxies (b2Fixture.cpp:121-137)
int World::CreateFixture(int bi, const Shape& shape, float density, float friction, float restitution,
                         int category, int mask, int group, bool sensor)
{
    Fixture fx;
    fx.body = bi;
    fx.shape = shape;
    fx.density = density;
    fx.friction = friction;
    fx.restitution = restitution;
    fx.category = (uint16_t)category;
    fx.mask = (uint16_t)mask;
    fx.group = (int16_t)group;
    fx.sensor = sensor;
    int id = (int)fixtures.size();
    fixtures.push_back(fx);
    Body& b = bodies[bi];
    if (b.flags & kBActive) {
        Fixture& f = fixtures[id];
        f.proxyCount = 1;
        ComputeAABB(f.shape, b.xf, &f.aabb);
        f.proxyId = bp.CreateProxy(f.aabb, id);
    }
    if (shape.chain == 2) {
        // a chain's next child: after the previous one, so the body's list visits a chain's children
        // in ascending order as b2Fixture::Synchronize does (b2Fixture.cpp:154-177)
        fixtures[id].next = fixtures[id - 1].next;
        fixtures[id - 1].next = id;
    } else {
        fixtures[id].next = b.fixtureList;
        b.fixtureList = id;
    }
    if (density > 0.0f) ResetMassData(bi);
    wflags |= 0x1; // e_newFixture
    return id;
}

// b2World::CreateJoint (Dynamics/b2World.cpp:212-269) + b2RevoluteJoint::b2RevoluteJoint (b2RevoluteJoint.cpp:44-63)
int World::CreateRevolute(int a, int b, const float* f, int fl)
{
    Joint j;
    j.bodyA = a; j.bodyB = b;
    j.localAnchorA = V(f[0], f[1]);
    j.localAnchorB = V(f[2], f[3]);
    j.referenceAngle = f[4];
    j.lowerAngle = f[5];
    j.upperAngle = f[6];
    j.motorSpeed = f[7];
    j.maxMotorTorque = f[8];
    j.enableLimit = (fl & 1) != 0;
    j.enableMotor = (fl & 2) != 0;
    j.collideConnected = (fl & 4) != 0;
    return LinkJoint(j, a, b);
}

// b2World::CreateJoint for a revolute, distance (b2DistanceJoint.cpp:52-63) or weld (b2WeldJoint.cpp:
// 48-58) definition; f as the C-ABI's gb_create_joints: revolute as CreateRevolute, distance
// localAnchorA, localAnchorB, length, frequencyHz, dampingRatio, weld localAnchorA, localAnchorB,
// referenceAngle, frequencyHz, dampingRatio; flags bit 4 collideConnected.
int World::CreateJoint(int type, int a, int b, const float* f, int fl)
{
    if (type == kRevoluteJoint) return CreateRevolute(a, b, f, fl);
    Joint j;
    j.type = type;
    j.bodyA = a; j.bodyB = b;
    j.localAnchorA = V(f[0], f[1]);
    j.localAnchorB = V(f[2], f[3]);
    if (type == kWheelJoint) {
        // b2WheelJoint::b2WheelJoint (b2WheelJoint.cpp): the axis as given, its normal b2Cross(1, axis)
        j.localXAxisA = V(f[4], f[5]);
        j.localYAxisA = Cross(1.0f, j.localXAxisA);
        j.maxMotorTorque = f[6];
        j.motorSpeed = f[7];
        j.frequencyHz = f[8];
        j.dampingRatio = f[9];
        j.enableMotor = (fl & 2) != 0;
    } else if (type == kMouseJoint) {
        // b2MouseJoint::b2MouseJoint (b2MouseJoint.cpp:33-52): body B's point under the target
        j.target = V(f[0], f[1]);
        j.localAnchorA = V(0.0f, 0.0f);
        j.localAnchorB = MulT(bodies[b].xf, j.target);
        j.maxForce = f[2];
        j.frequencyHz = f[3];
        j.dampingRatio = f[4];
    } else if (type == kPulleyJoint) {
        // b2PulleyJoint::b2PulleyJoint (b2PulleyJoint.cpp:53-69)
        j.groundAnchorA = V(f[0], f[1]);
        j.groundAnchorB = V(f[2], f[3]);
        j.localAnchorA = V(f[4], f[5]);
        j.localAnchorB = V(f[6], f[7]);
        j.lengthA = f[8];
        j.lengthB = f[9];
        j.ratio = f[10];
        j.pulleyConstant = f[8] + j.ratio * f[9];
    } else if (type == kGearJoint) {
        // b2GearJoint::b2GearJoint (b2GearJoint.cpp:49-136): f[0], f[1] the coupled joints, f[2] the
        // ratio; the joint's own bodies become the coupled joints' bodies B
        const Joint& j1 = joints[(int)f[0]];
        const Joint& j2 = joints[(int)f[1]];
        j.typeA = j1.type;
        j.typeB = j2.type;
        j.bodyC = j1.bodyA; j.bodyA = j1.bodyB;
        j.bodyD = j2.bodyA; j.bodyB = j2.bodyB;
        j.localAnchorC = j1.localAnchorA; j.localAnchorA = j1.localAnchorB;
        j.localAnchorD = j2.localAnchorA; j.localAnchorB = j2.localAnchorB;
        j.referenceAngle = j1.referenceAngle;
        j.referenceAngleB = j2.referenceAngle;
        const Body &A = bodies[j.bodyA], &B = bodies[j.bodyB], &Cb = bodies[j.bodyC], &Db = bodies[j.bodyD];
        float coordA, coordB;
        if (j1.type == kRevoluteJoint) {
            coordA = A.sweep.a - Cb.sweep.a - j.referenceAngle;
        } else {
            j.localAxisC = j1.localXAxisA;
            const Vec2 rel = MulT(Cb.xf.q, Mul(A.xf.q, j.localAnchorA) + (A.xf.p - Cb.xf.p));
            coordA = Dot(rel - j.localAnchorC, j.localAxisC);
        }
        if (j2.type == kRevoluteJoint) {
            coordB = B.sweep.a - Db.sweep.a - j.referenceAngleB;
        } else {
            j.localAxisD = j2.localXAxisA;
            const Vec2 rel = MulT(Db.xf.q, Mul(B.xf.q, j.localAnchorB) + (B.xf.p - Db.xf.p));
            coordB = Dot(rel - j.localAnchorD, j.localAxisD);
        }
        j.ratio = f[2];
        j.gearConstant = coordA + j.ratio * coordB;
    } else if (type == kRopeJoint) {
        j.maxLength = f[4];
    } else if (type == kFrictionJoint) {
        j.maxForce = f[4];
        j.maxTorque = f[5];
    } else if (type == kMotorJoint) {
        // b2MotorJoint::b2MotorJoint (b2MotorJoint.cpp): no anchors, the offsets in f[0..2]
        j.localAnchorA = V(0.0f, 0.0f);
        j.localAnchorB = V(0.0f, 0.0f);
        j.linearOffset = V(f[0], f[1]);
        j.angularOffset = f[2];
        j.maxForce = f[3];
        j.maxTorque = f[4];
        j.correctionFactor = f[5];
    } else if (type == kPrismaticJoint) {
        // b2PrismaticJoint::b2PrismaticJoint (b2PrismaticJoint.cpp:102-126)
        j.localXAxisA = V(f[4], f[5]);
        Normalize(j.localXAxisA);
        j.localYAxisA = Cross(1.0f, j.localXAxisA);
        j.referenceAngle = f[6];
        j.lowerAngle = f[7];
        j.upperAngle = f[8];
        j.maxMotorTorque = f[9];
        j.motorSpeed = f[10];
        j.enableLimit = (fl & 1) != 0;
        j.enableMotor = (fl & 2) != 0;
    } else {
        if (type == kDistanceJoint) j.length = f[4];
        else j.referenceAngle = f[4];
        j.frequencyHz = f[5];
        j.dampingRatio = f[6];
    }
    j.collideConnected = (fl & 4) != 0;
    return LinkJoint(j, a, b);
}

// b2World::CreateJoint (Dynamics/b2World.cpp:212-269): the joint list, both bodies' joint edges, and
// the filter flag on contacts between the bodies when they may not collide.
int World::LinkJoint(Joint& j, int a, int b)
{
    int id = (int)joints.size();
    j.prev = kNull;
    j.next = jointList;
    joints.push_back(j);
    if (jointList != kNull) joints[jointList].prev = id;
    jointList = id;
    ++jointCount;
    // edge 2*id is on bodyA's list (other = bodyB), 2*id+1 on bodyB's list (other = bodyA); the
    // joint's bodies (a gear joint's are not the definition's a, b, which the filter flag uses)
    for (int side = 0; side < 2; ++side) {
        Body& body = bodies[side == 0 ? j.bodyA : j.bodyB];
        int e = 2 * id + side;
        joints[id].ePrev[side] = kNull;
        joints[id].eNext[side] = body.jointList;
        if (body.jointList != kNull) joints[body.jointList >> 1].ePrev[body.jointList & 1] = e;
        body.jointList = e;
    }
    if (!j.collideConnected) {
        for (int e = bodies[b].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1])
            if (EdgeOther(e) == a) contacts[e >> 1].flags |= kCFilter;
    }
    return id;
}

int World::EdgeOther(int e) const
{
    const Contact& c = contacts[e >> 1];
    return (e & 1) == 0 ? fixtures[c.fB].body : fixtures[c.fA].body;
}
int World::JointEdgeOther(int e) const
{
    const Joint& j = joints[e >> 1];
    return (e & 1) == 0 ? j.bodyB : j.bodyA;
}

// b2Body::SetAwake (Dynamics/b2Body.h:625-645)
void World::SetAwake(int bi, bool flag)
{
    Body& b = bodies[bi];
    if (flag) {
        if ((b.flags & kBAwake) == 0) { b.flags |= kBAwake; b.sleepTime = 0.0f; }
    } else {
        b.flags &= ~kBAwake;
        b.sleepTime = 0.0f;
        b.v = V(0.0f, 0.0f);
        b.w = 0.0f;
        b.force = V(0.0f, 0.0f);
        b.torque = 0.0f;
    }
}

// b2Body::ShouldCollide (Dynamics/b2Body.cpp:354-375), called as bodyB->ShouldCollide(bodyA)
bool World::ShouldCollide(int self, int other) const
{
    if (bodies[self].type != kDynamic && bodies[other].type != kDynamic) return false;
    for (int e = bodies[self].jointList; e != kNull; e = joints[e >> 1].eNext[e & 1]) {
        if (JointEdgeOther(e) == other && !joints[e >> 1].collideConnected) return false;
    }
    return true;
}

// b2Body::SynchronizeTransform (Dynamics/b2Body.h:850-854)
void World::SynchronizeTransform(int bi)
{
    Body& b = bodies[bi];
    b.xf.q = RotOf(b.sweep.a);
    b.xf.p = b.sweep.c - Mul(b.xf.q, b.sweep.localCenter);
}

// b2Body::Advance (Dynamics/b2Body.h:856-864)
void World::Advance(int bi, float alpha)
{
    Body& b = bodies[bi];
    SweepAdvance(b.sweep, alpha);
    b.sweep.c = b.sweep.c0;
    b.sweep.a = b.sweep.a0;
    b.xf.q = RotOf(b.sweep.a);
    b.xf.p = b.sweep.c - Mul(b.xf.q, b.sweep.localCenter);
}

// b2Body::SynchronizeFixtures (Dynamics/b2Body.cpp:443-455) + b2Fixture::Synchronize (b2Fixture.cpp:154-177)
void World::SynchronizeFixtures(int bi)
{
    Body& b = bodies[bi];
    Xf xf1;
    xf1.q = RotOf(b.sweep.a0);
    xf1.p = b.sweep.c0 - Mul(xf1.q, b.sweep.localCenter);
    SynchronizeFixturesFrom(bi, xf1, b.xf);
}

// b2Fixture::Synchronize (Dynamics/b2Fixture.cpp:154-177) of every fixture of body bi from xf1 to xf2
void World::SynchronizeFixturesFrom(int bi, const Xf& xf1, const Xf& xf2)
{
    Body& b = bodies[bi];
    for (int f = b.fixtureList; f != kNull; f = fixtures[f].next) {
        Fixture& fx = fixtures[f];
        if (fx.proxyCount == 0) continue;
        AABB a1, a2;
        ComputeAABB(fx.shape, xf1, &a1);
        ComputeAABB(fx.shape, xf2, &a2);
        fx.aabb = Combine(a1, a2);
        Vec2 displacement = xf2.p - xf1.p;
        bp.MoveProxy(fx.proxyId, fx.aabb, displacement);
    }
}

// b2Body property changes between steps (prop: the C-ABI's GB_BODY_* code): SetType
// (Dynamics/b2Body.cpp:115-166), SetActive (:456-499), SetFixedRotation (:501-520), SetBullet,
// SetSleepingAllowed, SetLinearDamping, SetAngularDamping, SetGravityScale (b2Body.h:593-682).
void World::SetBodyProperty(int bi, int prop, const float* v)
{
    Body& b = bodies[bi];
    const bool flag = v[0] != 0.0f;
    auto destroyContacts = [&]() {
        for (int e = bodies[bi].contactList; e != kNull;) {
            const int c = e >> 1;
            e = contacts[c].eNext[e & 1];
            Destroy(c);
        }
        bodies[bi].contactList = kNull;
    };
    switch (prop) {
    case 0: {  // type
        const int type = (int)v[0];
        if (b.type == type) return;
        b.type = type;
        ResetMassData(bi);
        if (type == kStatic) {
            bodies[bi].v = V(0.0f, 0.0f);
            bodies[bi].w = 0.0f;
            bodies[bi].sweep.a0 = bodies[bi].sweep.a;
            bodies[bi].sweep.c0 = bodies[bi].sweep.c;
            SynchronizeFixtures(bi);
        }
        SetAwake(bi, true);
        bodies[bi].force = V(0.0f, 0.0f);
        bodies[bi].torque = 0.0f;
        destroyContacts();
        for (int f = bodies[bi].fixtureList; f != kNull; f = fixtures[f].next)
            if (fixtures[f].proxyCount > 0) bp.TouchProxy(fixtures[f].proxyId);
        return;
    }
    case 1: {  // active
        const bool active = (b.flags & kBActive) != 0;
        if (flag == active) return;
        if (flag) {
            b.flags |= kBActive;
            for (int f = b.fixtureList; f != kNull; f = fixtures[f].next) {
                Fixture& fx = fixtures[f];
                fx.proxyCount = 1;
                ComputeAABB(fx.shape, b.xf, &fx.aabb);
                fx.proxyId = bp.CreateProxy(fx.aabb, f);
            }
        } else {
            b.flags &= ~kBActive;
            for (int f = b.fixtureList; f != kNull; f = fixtures[f].next) {
                Fixture& fx = fixtures[f];
                if (fx.proxyCount > 0) bp.DestroyProxy(fx.proxyId);
                fx.proxyId = kNull;
                fx.proxyCount = 0;
            }
            destroyContacts();
        }
        return;
    }
    case 2: {  // fixed rotation
        const bool fixed = (b.flags & kBFixedRot) != 0;
        if (fixed == flag) return;
        if (flag) b.flags |= kBFixedRot;
        else b.flags &= ~kBFixedRot;
        b.w = 0.0f;
        ResetMassData(bi);
        return;
    }
    case 3:  // bullet
        if (flag) b.flags |= kBBullet;
        else b.flags &= ~kBBullet;
        return;
    case 4:  // sleeping allowed
        if (flag) {
            b.flags |= kBAutoSleep;
        } else {
            b.flags &= ~kBAutoSleep;
            SetAwake(bi, true);
        }
        return;
    case 5: b.linearDamping = v[0]; return;
    case 6: b.angularDamping = v[0]; return;
    case 7: b.gravityScale = v[0]; return;
    case 8: {  // SetMassData (b2Body.cpp:355-394): v = mass, center x, center y, rotational inertia
        if (b.type != kDynamic) return;
        b.invMass = 0.0f;
        b.I = 0.0f;
        b.invI = 0.0f;
        b.mass = v[0] <= 0.0f ? 1.0f : v[0];
        b.invMass = 1.0f / b.mass;
        const Vec2 center = V(v[1], v[2]);
        if (v[3] > 0.0f && (b.flags & kBFixedRot) == 0) {
            b.I = v[3] - b.mass * Dot(center, center);
            b.invI = 1.0f / b.I;
        }
        const Vec2 oldCenter = b.sweep.c;
        b.sweep.localCenter = center;
        b.sweep.c = Mul(b.xf, center);
        b.sweep.c0 = b.sweep.c;
        b.v = b.v + Cross(b.w, b.sweep.c - oldCenter);
        return;
    }
    case 9: ResetMassData(bi); return;  // b2Body::ResetMassData (b2Body.cpp:283-353)
    default: return;
    }
}

// Joint changes between steps (prop: the C-ABI's GB_JOINT_*), with the reference's wakes and limit
// impulse resets: b2RevoluteJoint::EnableMotor, SetMotorSpeed, SetMaxMotorTorque, EnableLimit,
// SetLimits (b2RevoluteJoint.cpp:419-483), the prismatic's (b2PrismaticJoint.cpp:546-604) and the
// wheel's (b2WheelJoint.cpp:377-396) counterparts, the spring, length, force and offset setters of the
// distance, weld, wheel, rope, friction, motor, gear and mouse joints (their headers; b2MotorJoint.cpp:
// 228-284). Returns 0, or 1 when the joint has no such property.
int World::SetJointProperty(int ji, int prop, const float* v)
{
    Joint& j = joints[ji];
    const int t = j.type;
    const bool motorised = t == kRevoluteJoint || t == kPrismaticJoint || t == kWheelJoint;
    const bool limited = t == kRevoluteJoint || t == kPrismaticJoint;
    const bool spring = t == kDistanceJoint || t == kWeldJoint || t == kWheelJoint || t == kMouseJoint;
    auto wake = [&]() {
        SetAwake(j.bodyA, true);
        SetAwake(j.bodyB, true);
    };
    switch (prop) {
    case 0: if (!motorised) return 1; wake(); j.motorSpeed = v[0]; return 0;
    case 1: if (!motorised) return 1; wake(); j.maxMotorTorque = v[0]; return 0;
    case 2: if (!motorised) return 1; wake(); j.enableMotor = v[0] != 0.0f; return 0;
    case 3: {
        if (!limited) return 1;
        const bool flag = v[0] != 0.0f;
        if (flag != j.enableLimit) {
            wake();
            j.enableLimit = flag;
            j.impulse[2] = 0.0f;
        }
        return 0;
    }
    case 4:
        if (!limited || !(v[0] <= v[1])) return 1;
        if (v[0] != j.lowerAngle || v[1] != j.upperAngle) {
            wake();
            j.impulse[2] = 0.0f;
            j.lowerAngle = v[0];
            j.upperAngle = v[1];
        }
        return 0;
    case 5: if (t != kDistanceJoint) return 1; j.length = v[0]; return 0;
    case 6: if (!spring) return 1; j.frequencyHz = v[0]; return 0;
    case 7: if (!spring) return 1; j.dampingRatio = v[0]; return 0;
    case 8: if (t != kRopeJoint) return 1; j.maxLength = v[0]; return 0;
    case 9: if (t != kFrictionJoint && t != kMotorJoint && t != kMouseJoint) return 1; j.maxForce = v[0]; return 0;
    case 10: if (t != kFrictionJoint && t != kMotorJoint) return 1; j.maxTorque = v[0]; return 0;
    case 11:
        if (t != kMotorJoint) return 1;
        if (v[0] != j.linearOffset.x || v[1] != j.linearOffset.y) {
            wake();
            j.linearOffset = V(v[0], v[1]);
        }
        return 0;
    case 12:
        if (t != kMotorJoint) return 1;
        if (v[0] != j.angularOffset) {
            wake();
            j.angularOffset = v[0];
        }
        return 0;
    case 13: if (t != kMotorJoint) return 1; j.correctionFactor = v[0]; return 0;
    case 14: if (t != kGearJoint) return 1; j.ratio = v[0]; return 0;
    default: return 1;
    }
}

// b2World::ShiftOrigin (b2World.cpp:1261-1282): body transforms and sweep centres, the mouse joint's
// target and the pulley's ground anchors (b2MouseJoint.cpp:222, b2PulleyJoint.cpp:347), and every
// node box of the broadphase tree (b2DynamicTree.cpp:773-781) move by -origin.
void World::ShiftOrigin(Vec2 o)
{
    for (int b = bodyList; b != kNull; b = bodies[b].next) {
        Body& x = bodies[b];
        x.xf.p = x.xf.p - o;
        x.sweep.c0 = x.sweep.c0 - o;
        x.sweep.c = x.sweep.c - o;
    }
    for (Joint& j : joints) {
        if (j.type == kMouseJoint) j.target = j.target - o;
        if (j.type == kPulleyJoint) {
            j.groundAnchorA = j.groundAnchorA - o;
            j.groundAnchorB = j.groundAnchorB - o;
        }
    }
    for (TreeNode& n : bp.tree.nodes) {
        n.aabb.lo = n.aabb.lo - o;
        n.aabb.hi = n.aabb.hi - o;
    }
}

// b2Fixture changes between steps (prop: the C-ABI's GB_FIXTURE_*): SetFriction, SetRestitution,
// SetDensity (b2Fixture.h:300-340), SetSensor (b2Fixture.cpp:418-425, wakes the body on a change),
// SetFilterData with Refilter (b2Fixture.cpp:181-214: the fixture's contacts flagged for filtering,
// its proxies touched). A chain (its first child's index) changes with all of its children.
void World::SetFixtureProperty(int f, int prop, const float* v)
{
    int last = f;
    const int body = fixtures[f].body;
    if (fixtures[f].shape.chain == 1)
        while (last + 1 < (int)fixtures.size() && fixtures[last + 1].body == body && fixtures[last + 1].shape.chain == 2)
            ++last;
    switch (prop) {
    case 0: for (int k = f; k <= last; ++k) fixtures[k].friction = v[0]; return;
    case 1: for (int k = f; k <= last; ++k) fixtures[k].restitution = v[0]; return;
    case 2: for (int k = f; k <= last; ++k) fixtures[k].density = v[0]; return;
    case 3: {
        const bool sensor = v[0] != 0.0f;
        if (sensor == fixtures[f].sensor) return;
        SetAwake(body, true);
        for (int k = f; k <= last; ++k) fixtures[k].sensor = sensor;
        return;
    }
    case 4: {
        for (int k = f; k <= last; ++k) {
            fixtures[k].category = (uint16_t)(int)v[0];
            fixtures[k].mask = (uint16_t)(int)v[1];
            fixtures[k].group = (int16_t)(int)v[2];
        }
        for (int e = bodies[body].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1]) {
            Contact& c = contacts[e >> 1];
            if ((c.fA >= f && c.fA <= last) || (c.fB >= f && c.fB <= last)) c.flags |= kCFilter;
        }
        for (int k = f; k <= last; ++k)
            if (fixtures[k].proxyCount > 0) bp.TouchProxy(fixtures[k].proxyId);
        return;
    }
    default: return;
    }
}

// b2Body state changes between steps: SetTransform (Dynamics/b2Body.cpp:419-441), SetLinearVelocity,
// SetAngularVelocity (b2Body.h:501-530), SetAwake (b2Body.h:635-655), ApplyForce, ApplyForceToCenter,
// ApplyTorque, ApplyLinearImpulse, ApplyAngularImpulse (b2Body.h:739-830). op: the C-ABI's GB_EDIT_*.
void World::ApplyEdit(int op, int bi, int wake, const float* v)
{
    if (op == 9) {
        // b2MouseJoint::SetTarget (b2MouseJoint.cpp:54-61); bi is the joint
        Joint& j = joints[bi];
        if ((bodies[j.bodyB].flags & kBAwake) == 0) SetAwake(j.bodyB, true);
        j.target = V(v[0], v[1]);
        return;
    }
    Body& b = bodies[bi];
    auto wakeOnRequest = [&]() {
        if (wake && (b.flags & kBAwake) == 0) SetAwake(bi, true);
    };
    switch (op) {
    case 0: {
        b.xf.q = RotOf(v[2]);
        b.xf.p = V(v[0], v[1]);
        b.sweep.c = Mul(b.xf, b.sweep.localCenter);
        b.sweep.a = v[2];
        b.sweep.c0 = b.sweep.c;
        b.sweep.a0 = v[2];
        SynchronizeFixturesFrom(bi, b.xf, b.xf);
        break;
    }
    case 1: {
        if (b.type == kStatic) break;
        const Vec2 vel = V(v[0], v[1]);
        if (Dot(vel, vel) > 0.0f) SetAwake(bi, true);
        b.v = vel;
        break;
    }
    case 2:
        if (b.type == kStatic) break;
        if (v[0] * v[0] > 0.0f) SetAwake(bi, true);
        b.w = v[0];
        break;
    case 3:
        SetAwake(bi, v[0] != 0.0f);
        break;
    case 4: case 5: case 6:
        if (b.type != kDynamic) break;
        wakeOnRequest();
        if ((b.flags & kBAwake) == 0) break;
        if (op == 6) {
            b.torque += v[0];
        } else {
            b.force = b.force + V(v[0], v[1]);
            if (op == 4) b.torque += Cross(V(v[2], v[3]) - b.sweep.c, V(v[0], v[1]));
        }
        break;
    case 7: case 8:
        if (b.type != kDynamic) break;
        wakeOnRequest();
        if ((b.flags & kBAwake) == 0) break;
        if (op == 7) {
            b.v = b.v + b.invMass * V(v[0], v[1]);
            b.w += b.invI * Cross(V(v[2], v[3]) - b.sweep.c, V(v[0], v[1]));
        } else {
            b.w += b.invI * v[0];
        }
        break;
    default:
        break;
    }
}

// ---------------------------------------------------------------- contact manager
// b2ContactManager::FindNewContacts (Dynamics/b2ContactManager.cpp:174-177) via UpdatePairs
void World::FindNewContacts()
{
    std::vector<Pair> list;
    bp.ComputePairs(list);
    for (const Pair& p : list) stepPairs.push_back(p);
    stepPairs.push_back(Pair{-1, -1});
    for (const Pair& p : list) AddPair(p.a, p.b);
}

static bool PrimaryOrder(int t1, int t2, bool* exists)
{
    // b2Contact::InitializeRegisters (Dynamics/Contacts/b2Contact.cpp:40-49): primary (A-type, B-type)
    // pairs are circle/circle, polygon/circle, polygon/polygon, edge/circle, edge/polygon.
    *exists = !(t1 == kEdge && t2 == kEdge);
    if (t1 == t2) return true;
    if (t1 == kPolygon && t2 == kCircle) return true;
    if (t1 == kEdge) return true;
    return false;
}

// b2ContactManager::AddPair (Dynamics/b2ContactManager.cpp:179-294)
void World::AddPair(int proxyA, int proxyB)
{
    int fixtureA = bp.tree.nodes[proxyA].user, fixtureB = bp.tree.nodes[proxyB].user;
    int bodyA = fixtures[fixtureA].body, bodyB = fixtures[fixtureB].body;
    if (bodyA == bodyB) return;
    for (int e = bodies[bodyB].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1]) {
        if (EdgeOther(e) == bodyA) {
            const Contact& c = contacts[e >> 1];
            if (c.fA == fixtureA && c.fB == fixtureB) return;
            if (c.fA == fixtureB && c.fB == fixtureA) return;
        }
    }
    if (!ShouldCollide(bodyB, bodyA)) return;
    const Fixture& fa = fixtures[fixtureA];
    const Fixture& fb = fixtures[fixtureB];
    if (!FilterShouldCollide(fixtureA, fixtureB)) return;
    bool exists;
    bool primary = PrimaryOrder(fa.shape.type, fb.shape.type, &exists);
    if (!exists) return;
    int fA = primary ? fixtureA : fixtureB, fB = primary ? fixtureB : fixtureA;
    int c;
    if (!freeContacts.empty()) { c = freeContacts.back(); freeContacts.pop_back(); contacts[c] = Contact(); }
    else { c = (int)contacts.size(); contacts.push_back(Contact()); }
    Contact& ct = contacts[c];
    ct.alive = true;
    ct.flags = kCEnabled;
    ct.fA = fA; ct.fB = fB;
    ct.m.pointCount = 0;
    ct.toiCount = 0;
    ct.friction = sqrtf(fixtures[fA].friction * fixtures[fB].friction);
    float ra = fixtures[fA].restitution, rb = fixtures[fB].restitution;
    ct.restitution = ra > rb ? ra : rb;
    ct.tangentSpeed = 0.0f;
    Link(c);
    if (!fixtures[fA].sensor && !fixtures[fB].sensor) {
        SetAwake(fixtures[fA].body, true);
        SetAwake(fixtures[fB].body, true);
    }
    ++contactCount;
}

// Prepend to the world list and both bodies' edge lists (b2ContactManager.cpp:255-290).
int World::Link(int c)
{
    Contact& ct = contacts[c];
    ct.prev = kNull;
    ct.next = contactList;
    if (contactList != kNull) contacts[contactList].prev = c;
    contactList = c;
    int bA = fixtures[ct.fA].body, bB = fixtures[ct.fB].body;
    for (int side = 0; side < 2; ++side) {
        Body& body = bodies[side == 0 ? bA : bB];
        int e = 2 * c + side;
        contacts[c].ePrev[side] = kNull;
        contacts[c].eNext[side] = body.contactList;
        if (body.contactList != kNull) contacts[body.contactList >> 1].ePrev[body.contactList & 1] = e;
        body.contactList = e;
    }
    return c;
}

// b2ContactManager::Destroy (Dynamics/b2ContactManager.cpp:39-105) + b2Contact::Destroy (b2Contact.cpp:102-123)
void World::Destroy(int c)
{
    Contact& ct = contacts[c];
    int bA = fixtures[ct.fA].body, bB = fixtures[ct.fB].body;
    if (ct.flags & kCTouching) {
        if (recordEvents) events.push_back(Event{1, ct.fA, ct.fB, 0, 0, 0, 0});
    }
    if (ct.prev != kNull) contacts[ct.prev].next = ct.next;
    if (ct.next != kNull) contacts[ct.next].prev = ct.prev;
    if (c == contactList) contactList = ct.next;
    for (int side = 0; side < 2; ++side) {
        int body = side == 0 ? bA : bB;
        int e = 2 * c + side;
        int pe = ct.ePrev[side], ne = ct.eNext[side];
        if (pe != kNull) contacts[pe >> 1].eNext[pe & 1] = ne;
        if (ne != kNull) contacts[ne >> 1].ePrev[ne & 1] = pe;
        if (bodies[body].contactList == e) bodies[body].contactList = ne;
    }
    if (ct.m.pointCount > 0 && !fixtures[ct.fA].sensor && !fixtures[ct.fB].sensor) {
        SetAwake(bA, true);
        SetAwake(bB, true);
    }
    ct.alive = false;
    freeContacts.push_back(c);
    --contactCount;
}

// b2Contact::Evaluate dispatch (Dynamics/Contacts/b2*Contact.cpp Evaluate)
void World::Evaluate(int c, Manifold* m)
{
    const Contact& ct = contacts[c];
    const Fixture& fa = fixtures[ct.fA];
    const Fixture& fb = fixtures[ct.fB];
    const Xf& xfA = bodies[fa.body].xf;
    const Xf& xfB = bodies[fb.body].xf;
    int ta = fa.shape.type, tb = fb.shape.type;
    if (ta == kCircle) CollideCircles(m, fa.shape, xfA, fb.shape, xfB);
    else if (ta == kPolygon && tb == kCircle) CollidePolygonAndCircle(m, fa.shape, xfA, fb.shape, xfB);
    else if (ta == kPolygon) CollidePolygons(m, fa.shape, xfA, fb.shape, xfB);
    else if (tb == kCircle) CollideEdgeAndCircle(m, fa.shape, xfA, fb.shape, xfB);
    else CollideEdgeAndPolygon(m, fa.shape, xfA, fb.shape, xfB);
}

// b2Contact::Update (Dynamics/Contacts/b2Contact.cpp:164-245). Sensors: overlap test via GJK.
void World::Update(int c)
{
    Contact& ct = contacts[c];
    Manifold old = ct.m;
    ct.flags |= kCEnabled;
    bool touching = false;
    bool wasTouching = (ct.flags & kCTouching) != 0;
    const Fixture& fa = fixtures[ct.fA];
    const Fixture& fb = fixtures[ct.fB];
    bool sensor = fa.sensor || fb.sensor;
    int bA = fa.body, bB = fb.body;
    if (sensor) {
        DistanceProxy pa, pb;
        ProxyOf(&pa, fa.shape);
        ProxyOf(&pb, fb.shape);
        SimplexCache cache;
        cache.count = 0;
        DistanceOutput out;
        Distance(&out, &cache, pa, bodies[bA].xf, pb, bodies[bB].xf, true);
        touching = out.distance < 10.0f * kEpsilon;
        ct.m.pointCount = 0;
    } else {
        Evaluate(c, &ct.m);
        touching = ct.m.pointCount > 0;
        for (int i = 0; i < ct.m.pointCount; ++i) {
            ManifoldPoint* mp2 = ct.m.points + i;
            mp2->normalImpulse = 0.0f;
            mp2->tangentImpulse = 0.0f;
            for (int j = 0; j < old.pointCount; ++j) {
                if (old.points[j].id == mp2->id) {
                    mp2->normalImpulse = old.points[j].normalImpulse;
                    mp2->tangentImpulse = old.points[j].tangentImpulse;
                    break;
                }
            }
        }
        if (touching != wasTouching) {
            SetAwake(bA, true);
            SetAwake(bB, true);
        }
    }
    if (touching) ct.flags |= kCTouching;
    else ct.flags &= ~kCTouching;
    if (recordEvents) {
        if (!wasTouching && touching) events.push_back(Event{0, ct.fA, ct.fB, 0, 0, 0, 0});
        if (wasTouching && !touching) events.push_back(Event{1, ct.fA, ct.fB, 0, 0, 0, 0});
        if (!sensor && touching) events.push_back(Event{2, ct.fA, ct.fB, 0, 0, 0, 0});
    }
    // a PreSolve listener's changes (b2ContactListener::PreSolve, called here in b2Contact::Update)
    if (!sensor && touching && !preSolveRule.empty()) {
        const int ra = ct.fA < (int)preSolveRule.size() ? preSolveRule[ct.fA] : 0;
        const int rb = ct.fB < (int)preSolveRule.size() ? preSolveRule[ct.fB] : 0;
        const int both = ra & rb;
        if (both & 1) ct.flags &= ~kCEnabled;
        if (both & 2) ct.friction = 0.0f;
        if (both & 4) ct.restitution = 0.9f;
    }
}

// b2ContactManager::Collide (Dynamics/b2ContactManager.cpp:107-172)
void World::Collide()
{
    int c = contactList;
    while (c != kNull) {
        Contact& ct = contacts[c];
        int bA = fixtures[ct.fA].body, bB = fixtures[ct.fB].body;
        if (ct.flags & kCFilter) {
            bool keep = ShouldCollide(bB, bA);
            if (keep) keep = FilterShouldCollide(ct.fA, ct.fB);
            if (!keep) { int nuke = c; c = ct.next; Destroy(nuke); continue; }
            ct.flags &= ~kCFilter;
        }
        bool activeA = bodies[bA].IsAwake() && bodies[bA].type != kStatic;
        bool activeB = bodies[bB].IsAwake() && bodies[bB].type != kStatic;
        if (!activeA && !activeB) { c = ct.next; continue; }
        bool overlap = bp.TestOverlap(fixtures[ct.fA].proxyId, fixtures[ct.fB].proxyId);
        if (!overlap) { int nuke = c; c = ct.next; Destroy(nuke); continue; }
        Update(c);
        c = contacts[c].next;
    }
}

// ---------------------------------------------------------------- contact solver
namespace {
struct Mat22 { Vec2 ex, ey; };
inline Vec2 MulM(const Mat22& A, Vec2 v) { return V(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y); }
// b2Mat22::GetInverse (Common/b2Math.h:185-197)
inline Mat22 Inverse(const Mat22& M)
{
    float a = M.ex.x, b = M.ey.x, c = M.ex.y, d = M.ey.y;
    Mat22 B;
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    B.ex.x = det * d; B.ey.x = -det * b;
    B.ex.y = -det * c; B.ey.y = det * a;
    return B;
}

struct VelPoint { Vec2 rA, rB; float normalImpulse, tangentImpulse, normalMass, tangentMass, velocityBias; };
struct VelConstraint {
    VelPoint points[2];
    Vec2 normal;
    Mat22 normalMass, K;
    int indexA, indexB;
    float invMassA, invMassB, invIA, invIB, friction, restitution, tangentSpeed;
    int pointCount, contactIndex;
};
struct PosConstraint {
    Vec2 localPoints[2], localNormal, localPoint;
    int indexA, indexB;
    float invMassA, invMassB;
    Vec2 localCenterA, localCenterB;
    float invIA, invIB;
    int type;
    float radiusA, radiusB;
    int pointCount;
};

// b2ContactSolver (Dynamics/Contacts/b2ContactSolver.cpp)
struct ContactSolver {
    World* w;
    StepInfo step;
    std::vector<VelConstraint> vcs;
    std::vector<PosConstraint> pcs;
    const int* contactIds;
    int count;
    Position* positions;
    Velocity* velocities;

    // b2ContactSolver::b2ContactSolver (b2ContactSolver.cpp:49-141)
    ContactSolver(World* world, const StepInfo& st, const int* ids, int n, Position* pos, Velocity* vel)
        : w(world), step(st), contactIds(ids), count(n), positions(pos), velocities(vel)
    {
        vcs.resize(n);
        pcs.resize(n);
        for (int i = 0; i < n; ++i) {
            const Contact& c = w->contacts[ids[i]];
            const Fixture& fa = w->fixtures[c.fA];
            const Fixture& fb = w->fixtures[c.fB];
            const Body& bA = w->bodies[fa.body];
            const Body& bB = w->bodies[fb.body];
            const Manifold& m = c.m;
            VelConstraint& vc = vcs[i];
            vc.friction = c.friction;
            vc.restitution = c.restitution;
            vc.tangentSpeed = c.tangentSpeed;
            vc.indexA = bA.islandIndex;
            vc.indexB = bB.islandIndex;
            vc.invMassA = bA.invMass; vc.invMassB = bB.invMass;
            vc.invIA = bA.invI; vc.invIB = bB.invI;
            vc.contactIndex = i;
            vc.pointCount = m.pointCount;
            vc.K = Mat22{V(0, 0), V(0, 0)};
            vc.normalMass = Mat22{V(0, 0), V(0, 0)};
            PosConstraint& pc = pcs[i];
            pc.indexA = bA.islandIndex; pc.indexB = bB.islandIndex;
            pc.invMassA = bA.invMass; pc.invMassB = bB.invMass;
            pc.localCenterA = bA.sweep.localCenter; pc.localCenterB = bB.sweep.localCenter;
            pc.invIA = bA.invI; pc.invIB = bB.invI;
            pc.localNormal = m.localNormal;
            pc.localPoint = m.localPoint;
            pc.pointCount = m.pointCount;
            pc.radiusA = fa.shape.radius;
            pc.radiusB = fb.shape.radius;
            pc.type = m.type;
            for (int j = 0; j < m.pointCount; ++j) {
                VelPoint& p = vc.points[j];
                if (step.warmStarting) {
                    p.normalImpulse = step.dtRatio * m.points[j].normalImpulse;
                    p.tangentImpulse = step.dtRatio * m.points[j].tangentImpulse;
                } else {
                    p.normalImpulse = 0.0f;
                    p.tangentImpulse = 0.0f;
                }
                p.rA = V(0, 0); p.rB = V(0, 0);
                p.normalMass = 0.0f; p.tangentMass = 0.0f; p.velocityBias = 0.0f;
                pc.localPoints[j] = m.points[j].localPoint;
            }
        }
    }

    // b2ContactSolver::InitializeVelocityConstraints (b2ContactSolver.cpp:143-252)
    void InitVelocity()
    {
        for (int i = 0; i < count; ++i) {
            VelConstraint& vc = vcs[i];
            PosConstraint& pc = pcs[i];
            float radiusA = pc.radiusA, radiusB = pc.radiusB;
            const Manifold& m = w->contacts[contactIds[vc.contactIndex]].m;
            int indexA = vc.indexA, indexB = vc.indexB;
            float mA = vc.invMassA, mB = vc.invMassB, iA = vc.invIA, iB = vc.invIB;
            Vec2 cA = positions[indexA].c; float aA = positions[indexA].a;
            Vec2 vA = velocities[indexA].v; float wA = velocities[indexA].w;
            Vec2 cB = positions[indexB].c; float aB = positions[indexB].a;
            Vec2 vB = velocities[indexB].v; float wB = velocities[indexB].w;
            Xf xfA, xfB;
            xfA.q = RotOf(aA);
            xfB.q = RotOf(aB);
            xfA.p = cA - Mul(xfA.q, pc.localCenterA);
            xfB.p = cB - Mul(xfB.q, pc.localCenterB);
            WorldManifold wm;
            WorldManifoldInit(&wm, &m, xfA, radiusA, xfB, radiusB);
            vc.normal = wm.normal;
            for (int j = 0; j < vc.pointCount; ++j) {
                VelPoint& p = vc.points[j];
                p.rA = wm.points[j] - cA;
                p.rB = wm.points[j] - cB;
                float rnA = Cross(p.rA, vc.normal), rnB = Cross(p.rB, vc.normal);
                float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
                p.normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
                Vec2 tangent = Cross(vc.normal, 1.0f);
                float rtA = Cross(p.rA, tangent), rtB = Cross(p.rB, tangent);
                float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
                p.tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
                p.velocityBias = 0.0f;
                float vRel = Dot(vc.normal, vB + Cross(wB, p.rB) - vA - Cross(wA, p.rA));
                if (vRel < -kVelocityThreshold) p.velocityBias = -vc.restitution * vRel;
            }
            if (vc.pointCount == 2) {
                VelPoint& p1 = vc.points[0];
                VelPoint& p2 = vc.points[1];
                float rn1A = Cross(p1.rA, vc.normal), rn1B = Cross(p1.rB, vc.normal);
                float rn2A = Cross(p2.rA, vc.normal), rn2B = Cross(p2.rB, vc.normal);
                float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
                float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
                float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
                const float k_maxConditionNumber = 1000.0f;
                if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
                    vc.K.ex = V(k11, k12);
                    vc.K.ey = V(k12, k22);
                    vc.normalMass = Inverse(vc.K);
                } else {
                    vc.pointCount = 1;
                }
            }
        }
    }

    // b2ContactSolver::WarmStart (b2ContactSolver.cpp:254-292)
    void WarmStart()
    {
        for (int i = 0; i < count; ++i) {
            VelConstraint& vc = vcs[i];
            int indexA = vc.indexA, indexB = vc.indexB;
            float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
            Vec2 vA = velocities[indexA].v; float wA = velocities[indexA].w;
            Vec2 vB = velocities[indexB].v; float wB = velocities[indexB].w;
            Vec2 normal = vc.normal, tangent = Cross(normal, 1.0f);
            for (int j = 0; j < vc.pointCount; ++j) {
                VelPoint& p = vc.points[j];
                Vec2 P = p.normalImpulse * normal + p.tangentImpulse * tangent;
                wA -= iA * Cross(p.rA, P);
                vA = vA - mA * P;
                wB += iB * Cross(p.rB, P);
                vB = vB + mB * P;
            }
            velocities[indexA].v = vA; velocities[indexA].w = wA;
            velocities[indexB].v = vB; velocities[indexB].w = wB;
        }
    }

    // b2ContactSolver::SolveVelocityConstraints (b2ContactSolver.cpp:294-605)
    void SolveVelocity()
    {
        for (int i = 0; i < count; ++i) {
            VelConstraint& vc = vcs[i];
            int indexA = vc.indexA, indexB = vc.indexB;
            float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
            int pointCount = vc.pointCount;
            Vec2 vA = velocities[indexA].v; float wA = velocities[indexA].w;
            Vec2 vB = velocities[indexB].v; float wB = velocities[indexB].w;
            Vec2 normal = vc.normal, tangent = Cross(normal, 1.0f);
            float friction = vc.friction;
            for (int j = 0; j < pointCount; ++j) {
                VelPoint& p = vc.points[j];
                Vec2 dv = vB + Cross(wB, p.rB) - vA - Cross(wA, p.rA);
                float vt = Dot(dv, tangent) - vc.tangentSpeed;
                float lambda = p.tangentMass * (-vt);
                float maxFriction = friction * p.normalImpulse;
                float newImpulse = Clamp(p.tangentImpulse + lambda, -maxFriction, maxFriction);
                lambda = newImpulse - p.tangentImpulse;
                p.tangentImpulse = newImpulse;
                Vec2 P = lambda * tangent;
                vA = vA - mA * P;
                wA -= iA * Cross(p.rA, P);
                vB = vB + mB * P;
                wB += iB * Cross(p.rB, P);
            }
            if (pointCount == 1) {
                VelPoint& p = vc.points[0];
                Vec2 dv = vB + Cross(wB, p.rB) - vA - Cross(wA, p.rA);
                float vn = Dot(dv, normal);
                float lambda = -p.normalMass * (vn - p.velocityBias);
                float newImpulse = Max(p.normalImpulse + lambda, 0.0f);
                lambda = newImpulse - p.normalImpulse;
                p.normalImpulse = newImpulse;
                Vec2 P = lambda * normal;
                vA = vA - mA * P;
                wA -= iA * Cross(p.rA, P);
                vB = vB + mB * P;
                wB += iB * Cross(p.rB, P);
            } else {
                VelPoint& cp1 = vc.points[0];
                VelPoint& cp2 = vc.points[1];
                Vec2 a = V(cp1.normalImpulse, cp2.normalImpulse);
                Vec2 dv1 = vB + Cross(wB, cp1.rB) - vA - Cross(wA, cp1.rA);
                Vec2 dv2 = vB + Cross(wB, cp2.rB) - vA - Cross(wA, cp2.rA);
                float vn1 = Dot(dv1, normal), vn2 = Dot(dv2, normal);
                Vec2 b;
                b.x = vn1 - cp1.velocityBias;
                b.y = vn2 - cp2.velocityBias;
                b = b - MulM(vc.K, a);
                Vec2 x;
                bool solved = false;
                // Total enumeration of the 2-point LCP (b2ContactSolver.cpp:420-600)
                x = -MulM(vc.normalMass, b);
                if (x.x >= 0.0f && x.y >= 0.0f) solved = true;
                if (!solved) {
                    x.x = -cp1.normalMass * b.x;
                    x.y = 0.0f;
                    vn2 = vc.K.ex.y * x.x + b.y;
                    if (x.x >= 0.0f && vn2 >= 0.0f) solved = true;
                }
                if (!solved) {
                    x.x = 0.0f;
                    x.y = -cp2.normalMass * b.y;
                    vn1 = vc.K.ey.x * x.y + b.x;
                    if (x.y >= 0.0f && vn1 >= 0.0f) solved = true;
                }
                if (!solved) {
                    x.x = 0.0f;
                    x.y = 0.0f;
                    vn1 = b.x;
                    vn2 = b.y;
                    if (vn1 >= 0.0f && vn2 >= 0.0f) solved = true;
                }
                if (solved) {
                    Vec2 d = x - a;
                    Vec2 P1 = d.x * normal, P2 = d.y * normal;
                    vA = vA - mA * (P1 + P2);
                    wA -= iA * (Cross(cp1.rA, P1) + Cross(cp2.rA, P2));
                    vB = vB + mB * (P1 + P2);
                    wB += iB * (Cross(cp1.rB, P1) + Cross(cp2.rB, P2));
                    cp1.normalImpulse = x.x;
                    cp2.normalImpulse = x.y;
                }
            }
            velocities[indexA].v = vA; velocities[indexA].w = wA;
            velocities[indexB].v = vB; velocities[indexB].w = wB;
        }
    }

    // b2ContactSolver::StoreImpulses (b2ContactSolver.cpp:607-620)
    void StoreImpulses()
    {
        for (int i = 0; i < count; ++i) {
            const VelConstraint& vc = vcs[i];
            Manifold& m = w->contacts[contactIds[vc.contactIndex]].m;
            for (int j = 0; j < vc.pointCount; ++j) {
                m.points[j].normalImpulse = vc.points[j].normalImpulse;
                m.points[j].tangentImpulse = vc.points[j].tangentImpulse;
            }
        }
    }

    // b2PositionSolverManifold::Initialize (b2ContactSolver.cpp:623-672)
    static void PSM(const PosConstraint& pc, const Xf& xfA, const Xf& xfB, int index, Vec2* normal, Vec2* point, float* separation)
    {
        switch (pc.type) {
        case kCircles: {
            Vec2 pointA = Mul(xfA, pc.localPoint);
            Vec2 pointB = Mul(xfB, pc.localPoints[0]);
            *normal = pointB - pointA;
            Normalize(*normal);
            *point = 0.5f * (pointA + pointB);
            *separation = Dot(pointB - pointA, *normal) - pc.radiusA - pc.radiusB;
            break;
        }
        case kFaceA: {
            *normal = Mul(xfA.q, pc.localNormal);
            Vec2 planePoint = Mul(xfA, pc.localPoint);
            Vec2 clipPoint = Mul(xfB, pc.localPoints[index]);
            *separation = Dot(clipPoint - planePoint, *normal) - pc.radiusA - pc.radiusB;
            *point = clipPoint;
            break;
        }
        default: {
            *normal = Mul(xfB.q, pc.localNormal);
            Vec2 planePoint = Mul(xfB, pc.localPoint);
            Vec2 clipPoint = Mul(xfA, pc.localPoints[index]);
            *separation = Dot(clipPoint - planePoint, *normal) - pc.radiusA - pc.radiusB;
            *point = clipPoint;
            *normal = -*normal;
            break;
        }
        }
    }

    // b2ContactSolver::SolvePositionConstraints (b2ContactSolver.cpp:674-751) and
    // SolveTOIPositionConstraints (:753-836): toi == true uses the TOI Baumgarte, the TOI body masks
    // and the -1.5 slop acceptance.
    bool SolvePosition(bool toi, int toiA, int toiB)
    {
        float minSeparation = 0.0f;
        for (int i = 0; i < count; ++i) {
            const PosConstraint& pc = pcs[i];
            int indexA = pc.indexA, indexB = pc.indexB;
            Vec2 localCenterA = pc.localCenterA, localCenterB = pc.localCenterB;
            float mA, iA, mB, iB;
            if (!toi) { mA = pc.invMassA; iA = pc.invIA; mB = pc.invMassB; iB = pc.invIB; }
            else {
                mA = 0.0f; iA = 0.0f; mB = 0.0f; iB = 0.0f;
                if (indexA == toiA || indexA == toiB) { mA = pc.invMassA; iA = pc.invIA; }
                if (indexB == toiA || indexB == toiB) { mB = pc.invMassB; iB = pc.invIB; }
            }
            int pointCount = pc.pointCount;
            Vec2 cA = positions[indexA].c; float aA = positions[indexA].a;
            Vec2 cB = positions[indexB].c; float aB = positions[indexB].a;
            for (int j = 0; j < pointCount; ++j) {
                Xf xfA, xfB;
                xfA.q = RotOf(aA);
                xfB.q = RotOf(aB);
                xfA.p = cA - Mul(xfA.q, localCenterA);
                xfB.p = cB - Mul(xfB.q, localCenterB);
                Vec2 normal, point;
                float separation;
                PSM(pc, xfA, xfB, j, &normal, &point, &separation);
                Vec2 rA = point - cA, rB = point - cB;
                minSeparation = Min(minSeparation, separation);
                float C = toi ? Clamp(kToiBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f)
                              : Clamp(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
                float rnA = Cross(rA, normal), rnB = Cross(rB, normal);
                float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
                float impulse = K > 0.0f ? -C / K : 0.0f;
                Vec2 P = impulse * normal;
                cA = cA - mA * P;
                aA -= iA * Cross(rA, P);
                cB = cB + mB * P;
                aB += iB * Cross(rB, P);
            }
            positions[indexA].c = cA; positions[indexA].a = aA;
            positions[indexB].c = cB; positions[indexB].a = aB;
        }
        return toi ? minSeparation >= -1.5f * kLinearSlop : minSeparation >= -3.0f * kLinearSlop;
    }

    std::vector<float> ReportImpulses(int i) const
    {
        std::vector<float> r(4, 0.0f);
        for (int j = 0; j < vcs[i].pointCount; ++j) { r[j] = vcs[i].points[j].normalImpulse; r[2 + j] = vcs[i].points[j].tangentImpulse; }
        return r;
    }
};

// ---------------------------------------------------------------- revolute joint
inline Vec2 MulM33x(const float* m, Vec2 v)
{
    return V(m[0] * v.x + m[3] * v.y, m[1] * v.x + m[4] * v.y);
}

// b2RevoluteJoint::InitVelocityConstraints (Dynamics/Joints/b2RevoluteJoint.cpp:66-183)
void RevInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    float aA = pos[j.indexA].a;
    Vec2 vA = vel[j.indexA].v; float wA = vel[j.indexA].w;
    float aB = pos[j.indexB].a;
    Vec2 vB = vel[j.indexB].v; float wB = vel[j.indexB].w;
    Rot qA = RotOf(aA), qB = RotOf(aB);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    bool fixedRotation = (iA + iB == 0.0f);
    float* M = j.mass;
    M[0] = mA + mB + j.rA.y * j.rA.y * iA + j.rB.y * j.rB.y * iB;
    M[3] = -j.rA.y * j.rA.x * iA - j.rB.y * j.rB.x * iB;
    M[6] = -j.rA.y * iA - j.rB.y * iB;
    M[1] = M[3];
    M[4] = mA + mB + j.rA.x * j.rA.x * iA + j.rB.x * j.rB.x * iB;
    M[7] = j.rA.x * iA + j.rB.x * iB;
    M[2] = M[6];
    M[5] = M[7];
    M[8] = iA + iB;
    j.motorMass = iA + iB;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    if (!j.enableMotor || fixedRotation) j.motorImpulse = 0.0f;
    if (j.enableLimit && !fixedRotation) {
        float jointAngle = aB - aA - j.referenceAngle;
        if (Abs(j.upperAngle - j.lowerAngle) < 2.0f * kAngularSlop) j.limitState = 3;
        else if (jointAngle <= j.lowerAngle) {
            if (j.limitState != 1) j.impulse[2] = 0.0f;
            j.limitState = 1;
        } else if (jointAngle >= j.upperAngle) {
            if (j.limitState != 2) j.impulse[2] = 0.0f;
            j.limitState = 2;
        } else {
            j.limitState = 0;
            j.impulse[2] = 0.0f;
        }
    } else {
        j.limitState = 0;
    }
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio; j.impulse[1] *= step.dtRatio; j.impulse[2] *= step.dtRatio;
        j.motorImpulse *= step.dtRatio;
        Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.motorImpulse + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.motorImpulse + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
        j.motorImpulse = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// forward declarations of the joint kinds other than revolute (below)
void DistInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void DistSolveVelocity(Joint& j, Velocity* vel);
bool DistSolvePosition(Joint& j, Position* pos);
void WeldInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void WeldSolveVelocity(Joint& j, Velocity* vel);
bool WeldSolvePosition(Joint& j, Position* pos);
void PrisInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void PrisSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel);
bool PrisSolvePosition(Joint& j, Position* pos);
void WheelInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void WheelSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel);
bool WheelSolvePosition(Joint& j, Position* pos);
void RopeInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void RopeSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel);
bool RopeSolvePosition(Joint& j, Position* pos);
void FrictionMotorInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void MouseInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void MouseSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel);
void PulleyInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void GearInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel);
void GearSolveVelocity(Joint& j, Velocity* vel);
bool GearSolvePosition(Joint& j, Position* pos);
void PulleySolveVelocity(Joint& j, Velocity* vel);
bool PulleySolvePosition(Joint& j, Position* pos);
void FrictionMotorSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel);

// b2Mat33::Solve33 / Solve22 (Common/b2Math.cpp:24-56)
inline void Solve33(const float* M, const float* b, float* x)
{
    // columns ex = M[0..2], ey = M[3..5], ez = M[6..8]
    auto cross3 = [](const float* a, const float* c, float* o) {
        o[0] = a[1] * c[2] - a[2] * c[1];
        o[1] = a[2] * c[0] - a[0] * c[2];
        o[2] = a[0] * c[1] - a[1] * c[0];
    };
    auto dot3 = [](const float* a, const float* c) { return a[0] * c[0] + a[1] * c[1] + a[2] * c[2]; };
    float t[3];
    cross3(M + 3, M + 6, t);
    float det = dot3(M, t);
    if (det != 0.0f) det = 1.0f / det;
    x[0] = det * dot3(b, t);
    cross3(b, M + 6, t);
    x[1] = det * dot3(M, t);
    cross3(M + 3, b, t);
    x[2] = det * dot3(M, t);
}
inline Vec2 Solve22(const float* M, Vec2 b)
{
    float a11 = M[0], a12 = M[3], a21 = M[1], a22 = M[4];
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = 1.0f / det;
    return V(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}

// b2RevoluteJoint::SolveVelocityConstraints (b2RevoluteJoint.cpp:185-291)
void RevSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v; float wA = vel[j.indexA].w;
    Vec2 vB = vel[j.indexB].v; float wB = vel[j.indexB].w;
    float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    bool fixedRotation = (iA + iB == 0.0f);
    if (j.enableMotor && j.limitState != 3 && !fixedRotation) {
        float Cdot = wB - wA - j.motorSpeed;
        float impulse = -j.motorMass * Cdot;
        float oldImpulse = j.motorImpulse;
        float maxImpulse = step.dt * j.maxMotorTorque;
        j.motorImpulse = Clamp(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if (j.enableLimit && j.limitState != 0 && !fixedRotation) {
        Vec2 Cdot1 = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        float Cdot2 = wB - wA;
        float Cdot[3] = {Cdot1.x, Cdot1.y, Cdot2};
        float imp[3];
        Solve33(j.mass, Cdot, imp);
        imp[0] = -imp[0]; imp[1] = -imp[1]; imp[2] = -imp[2];
        if (j.limitState == 3) {
            j.impulse[0] += imp[0]; j.impulse[1] += imp[1]; j.impulse[2] += imp[2];
        } else if (j.limitState == 1 || j.limitState == 2) {
            float newImpulse = j.impulse[2] + imp[2];
            bool clampIt = j.limitState == 1 ? newImpulse < 0.0f : newImpulse > 0.0f;
            if (clampIt) {
                Vec2 rhs = -Cdot1 + j.impulse[2] * V(j.mass[6], j.mass[7]);
                Vec2 reduced = Solve22(j.mass, rhs);
                imp[0] = reduced.x;
                imp[1] = reduced.y;
                imp[2] = -j.impulse[2];
                j.impulse[0] += reduced.x;
                j.impulse[1] += reduced.y;
                j.impulse[2] = 0.0f;
            } else {
                j.impulse[0] += imp[0]; j.impulse[1] += imp[1]; j.impulse[2] += imp[2];
            }
        }
        Vec2 P = V(imp[0], imp[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + imp[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + imp[2]);
    } else {
        Vec2 Cdot = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        Vec2 impulse = Solve22(j.mass, -Cdot);
        j.impulse[0] += impulse.x;
        j.impulse[1] += impulse.y;
        vA = vA - mA * impulse;
        wA -= iA * Cross(j.rA, impulse);
        vB = vB + mB * impulse;
        wB += iB * Cross(j.rB, impulse);
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2RevoluteJoint::SolvePositionConstraints (b2RevoluteJoint.cpp:293-380)
bool RevSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c; float aA = pos[j.indexA].a;
    Vec2 cB = pos[j.indexB].c; float aB = pos[j.indexB].a;
    float angularError = 0.0f, positionError = 0.0f;
    bool fixedRotation = (j.invIA + j.invIB == 0.0f);
    if (j.enableLimit && j.limitState != 0 && !fixedRotation) {
        float angle = aB - aA - j.referenceAngle;
        float limitImpulse = 0.0f;
        if (j.limitState == 3) {
            float C = Clamp(angle - j.lowerAngle, -kMaxAngularCorrection, kMaxAngularCorrection);
            limitImpulse = -j.motorMass * C;
            angularError = Abs(C);
        } else if (j.limitState == 1) {
            float C = angle - j.lowerAngle;
            angularError = -C;
            C = Clamp(C + kAngularSlop, -kMaxAngularCorrection, 0.0f);
            limitImpulse = -j.motorMass * C;
        } else if (j.limitState == 2) {
            float C = angle - j.upperAngle;
            angularError = C;
            C = Clamp(C - kAngularSlop, 0.0f, kMaxAngularCorrection);
            limitImpulse = -j.motorMass * C;
        }
        aA -= j.invIA * limitImpulse;
        aB += j.invIB * limitImpulse;
    }
    {
        Rot qA = RotOf(aA), qB = RotOf(aB);
        Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
        Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
        Vec2 C = cB + rB - cA - rA;
        positionError = Length(C);
        float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
        float K[9] = {0};
        K[0] = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
        K[1] = -iA * rA.x * rA.y - iB * rB.x * rB.y;
        K[3] = K[1];
        K[4] = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
        Vec2 impulse = -Solve22(K, C);
        cA = cA - mA * impulse;
        aA -= iA * Cross(rA, impulse);
        cB = cB + mB * impulse;
        aB += iB * Cross(rB, impulse);
    }
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}

// ---------------------------------------------------------------- distance joint
// b2DistanceJoint::InitVelocityConstraints (Dynamics/Joints/b2DistanceJoint.cpp:65-158)
void DistInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    j.u = cB + j.rB - cA - j.rA;
    const float length = Length(j.u);
    if (length > kLinearSlop) {
        j.u.x *= 1.0f / length;
        j.u.y *= 1.0f / length;
    } else {
        j.u = V(0.0f, 0.0f);
    }
    const float crAu = Cross(j.rA, j.u), crBu = Cross(j.rB, j.u);
    float invMass = j.invMassA + j.invIA * crAu * crAu + j.invMassB + j.invIB * crBu * crBu;
    j.motorMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    if (j.frequencyHz > 0.0f) {
        const float C = length - j.length;
        const float omega = 2.0f * kPi * j.frequencyHz;
        const float d = 2.0f * j.motorMass * j.dampingRatio * omega;
        const float k = j.motorMass * omega * omega;
        const float h = step.dt;
        j.gamma = h * (d + h * k);
        j.gamma = j.gamma != 0.0f ? 1.0f / j.gamma : 0.0f;
        j.bias = C * h * k * j.gamma;
        invMass += j.gamma;
        j.motorMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    } else {
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio;
        const Vec2 P = j.impulse[0] * j.u;
        vA = vA - j.invMassA * P;
        wA -= j.invIA * Cross(j.rA, P);
        vB = vB + j.invMassB * P;
        wB += j.invIB * Cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2DistanceJoint::SolveVelocityConstraints (b2DistanceJoint.cpp:160-185)
void DistSolveVelocity(Joint& j, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Vec2 vpA = vA + Cross(wA, j.rA);
    const Vec2 vpB = vB + Cross(wB, j.rB);
    const float Cdot = Dot(j.u, vpB - vpA);
    const float impulse = -j.motorMass * (Cdot + j.bias + j.gamma * j.impulse[0]);
    j.impulse[0] += impulse;
    const Vec2 P = impulse * j.u;
    vA = vA - j.invMassA * P;
    wA -= j.invIA * Cross(j.rA, P);
    vB = vB + j.invMassB * P;
    wB += j.invIB * Cross(j.rB, P);
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2DistanceJoint::SolvePositionConstraints (b2DistanceJoint.cpp:187-226)
bool DistSolvePosition(Joint& j, Position* pos)
{
    if (j.frequencyHz > 0.0f) return true;
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    Vec2 u = cB + rB - cA - rA;
    const float length = Normalize(u);
    float C = length - j.length;
    C = Clamp(C, -kMaxLinearCorrection, kMaxLinearCorrection);
    const float impulse = -j.motorMass * C;
    const Vec2 P = impulse * u;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * Cross(rA, P);
    cB = cB + j.invMassB * P;
    aB += j.invIB * Cross(rB, P);
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return Abs(C) < kLinearSlop;
}

// ---------------------------------------------------------------- weld joint
// K of b2WeldJoint (b2WeldJoint.cpp:95-105 and 245-254), columns ex = K[0..2], ey = K[3..5], ez = K[6..8]
void WeldK(const Joint& j, Vec2 rA, Vec2 rB, float* K)
{
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    K[0] = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
    K[3] = -rA.y * rA.x * iA - rB.y * rB.x * iB;
    K[6] = -rA.y * iA - rB.y * iB;
    K[1] = K[3];
    K[4] = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
    K[7] = rA.x * iA + rB.x * iB;
    K[2] = K[6];
    K[5] = K[7];
    K[8] = iA + iB;
}

// b2Mat33::GetInverse22 (Common/b2Math.cpp:59-72): the 2x2 block's inverse, the rest zero
void Inverse22(const float* K, float* M)
{
    const float a = K[0], b = K[3], c = K[1], d = K[4];
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    M[0] = det * d; M[3] = -det * b; M[2] = 0.0f;
    M[1] = -det * c; M[4] = det * a; M[5] = 0.0f;
    M[6] = 0.0f; M[7] = 0.0f; M[8] = 0.0f;
}

// b2Mat33::GetSymInverse33 (Common/b2Math.cpp:74-97)
void SymInverse33(const float* K, float* M)
{
    const float cx = K[4] * K[8] - K[5] * K[7], cy = K[5] * K[6] - K[3] * K[8], cz = K[3] * K[7] - K[4] * K[6];
    float det = K[0] * cx + K[1] * cy + K[2] * cz;
    if (det != 0.0f) det = 1.0f / det;
    const float a11 = K[0], a12 = K[3], a13 = K[6];
    const float a22 = K[4], a23 = K[7];
    const float a33 = K[8];
    M[0] = det * (a22 * a33 - a23 * a23);
    M[1] = det * (a13 * a23 - a12 * a33);
    M[2] = det * (a12 * a23 - a13 * a22);
    M[3] = M[1];
    M[4] = det * (a11 * a33 - a13 * a13);
    M[5] = det * (a13 * a12 - a11 * a23);
    M[6] = M[2];
    M[7] = M[5];
    M[8] = det * (a11 * a22 - a12 * a12);
}

// b2WeldJoint::InitVelocityConstraints (Dynamics/Joints/b2WeldJoint.cpp:60-169)
void WeldInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float K[9];
    WeldK(j, j.rA, j.rB, K);
    if (j.frequencyHz > 0.0f) {
        Inverse22(K, j.mass);
        float invM = iA + iB;
        const float m = invM > 0.0f ? 1.0f / invM : 0.0f;
        const float C = aB - aA - j.referenceAngle;
        const float omega = 2.0f * kPi * j.frequencyHz;
        const float d = 2.0f * m * j.dampingRatio * omega;
        const float k = m * omega * omega;
        const float h = step.dt;
        j.gamma = h * (d + h * k);
        j.gamma = j.gamma != 0.0f ? 1.0f / j.gamma : 0.0f;
        j.bias = C * h * k * j.gamma;
        invM += j.gamma;
        j.mass[8] = invM != 0.0f ? 1.0f / invM : 0.0f;
    } else if (K[8] == 0.0f) {
        Inverse22(K, j.mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    } else {
        SymInverse33(K, j.mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio; j.impulse[1] *= step.dtRatio; j.impulse[2] *= step.dtRatio;
        const Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2WeldJoint::SolveVelocityConstraints (b2WeldJoint.cpp:171-227)
void WeldSolveVelocity(Joint& j, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float* M = j.mass;
    if (j.frequencyHz > 0.0f) {
        const float Cdot2 = wB - wA;
        const float impulse2 = -M[8] * (Cdot2 + j.bias + j.gamma * j.impulse[2]);
        j.impulse[2] += impulse2;
        wA -= iA * impulse2;
        wB += iB * impulse2;
        const Vec2 Cdot1 = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        const Vec2 impulse1 = -MulM33x(M, Cdot1);
        j.impulse[0] += impulse1.x;
        j.impulse[1] += impulse1.y;
        const Vec2 P = impulse1;
        vA = vA - mA * P;
        wA -= iA * Cross(j.rA, P);
        vB = vB + mB * P;
        wB += iB * Cross(j.rB, P);
    } else {
        const Vec2 Cdot1 = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        const float Cdot2 = wB - wA;
        // b2Mul(b2Mat33, b2Vec3) = Cdot.x * ex + Cdot.y * ey + Cdot.z * ez
        const float ix = -((Cdot1.x * M[0] + Cdot1.y * M[3]) + Cdot2 * M[6]);
        const float iy = -((Cdot1.x * M[1] + Cdot1.y * M[4]) + Cdot2 * M[7]);
        const float iz = -((Cdot1.x * M[2] + Cdot1.y * M[5]) + Cdot2 * M[8]);
        j.impulse[0] += ix;
        j.impulse[1] += iy;
        j.impulse[2] += iz;
        const Vec2 P = V(ix, iy);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + iz);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + iz);
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2WeldJoint::SolvePositionConstraints (b2WeldJoint.cpp:229-316)
bool WeldSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    float K[9];
    WeldK(j, rA, rB, K);
    float positionError, angularError;
    if (j.frequencyHz > 0.0f) {
        const Vec2 C1 = cB + rB - cA - rA;
        positionError = Length(C1);
        angularError = 0.0f;
        const Vec2 P = -Solve22(K, C1);
        cA = cA - mA * P;
        aA -= iA * Cross(rA, P);
        cB = cB + mB * P;
        aB += iB * Cross(rB, P);
    } else {
        const Vec2 C1 = cB + rB - cA - rA;
        const float C2 = aB - aA - j.referenceAngle;
        positionError = Length(C1);
        angularError = Abs(C2);
        float imp[3];
        if (K[8] > 0.0f) {
            const float Cv[3] = {C1.x, C1.y, C2};
            Solve33(K, Cv, imp);
            imp[0] = -imp[0]; imp[1] = -imp[1]; imp[2] = -imp[2];
        } else {
            const Vec2 i2 = -Solve22(K, C1);
            imp[0] = i2.x; imp[1] = i2.y; imp[2] = 0.0f;
        }
        const Vec2 P = V(imp[0], imp[1]);
        cA = cA - mA * P;
        aA -= iA * (Cross(rA, P) + imp[2]);
        cB = cB + mB * P;
        aB += iB * (Cross(rB, P) + imp[2]);
    }
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}


// ---------------------------------------------------------------- prismatic joint
// b2PrismaticJoint::InitVelocityConstraints (Dynamics/Joints/b2PrismaticJoint.cpp:128-266)
void PrisInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = (cB - cA) + rB - rA;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    j.u = Mul(qA, j.localXAxisA);
    j.a1 = Cross(d + rA, j.u);
    j.a2 = Cross(rB, j.u);
    j.motorMass = mA + mB + iA * j.a1 * j.a1 + iB * j.a2 * j.a2;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    j.perp = Mul(qA, j.localYAxisA);
    j.s1 = Cross(d + rA, j.perp);
    j.s2 = Cross(rB, j.perp);
    float* K = j.mass;
    K[0] = mA + mB + iA * j.s1 * j.s1 + iB * j.s2 * j.s2;
    K[1] = iA * j.s1 + iB * j.s2;
    K[2] = iA * j.s1 * j.a1 + iB * j.s2 * j.a2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    K[4] = k22;
    K[5] = iA * j.a1 + iB * j.a2;
    K[8] = mA + mB + iA * j.a1 * j.a1 + iB * j.a2 * j.a2;
    K[3] = K[1]; K[6] = K[2]; K[7] = K[5];
    if (j.enableLimit) {
        const float translation = Dot(j.u, d);
        if (Abs(j.upperAngle - j.lowerAngle) < 2.0f * kLinearSlop) {
            j.limitState = 3;
        } else if (translation <= j.lowerAngle) {
            if (j.limitState != 1) { j.limitState = 1; j.impulse[2] = 0.0f; }
        } else if (translation >= j.upperAngle) {
            if (j.limitState != 2) { j.limitState = 2; j.impulse[2] = 0.0f; }
        } else {
            j.limitState = 0;
            j.impulse[2] = 0.0f;
        }
    } else {
        j.limitState = 0;
        j.impulse[2] = 0.0f;
    }
    if (!j.enableMotor) j.motorImpulse = 0.0f;
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio; j.impulse[1] *= step.dtRatio; j.impulse[2] *= step.dtRatio;
        j.motorImpulse *= step.dtRatio;
        const Vec2 P = j.impulse[0] * j.perp + (j.motorImpulse + j.impulse[2]) * j.u;
        const float LA = j.impulse[0] * j.s1 + j.impulse[1] + (j.motorImpulse + j.impulse[2]) * j.a1;
        const float LB = j.impulse[0] * j.s2 + j.impulse[1] + (j.motorImpulse + j.impulse[2]) * j.a2;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
        j.motorImpulse = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2PrismaticJoint::SolveVelocityConstraints (b2PrismaticJoint.cpp:268-363)
void PrisSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    if (j.enableMotor && j.limitState != 3) {
        const float Cdot = Dot(j.u, vB - vA) + j.a2 * wB - j.a1 * wA;
        float impulse = j.motorMass * (j.motorSpeed - Cdot);
        const float oldImpulse = j.motorImpulse;
        const float maxImpulse = step.dt * j.maxMotorTorque;
        j.motorImpulse = Clamp(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        const Vec2 P = impulse * j.u;
        const float LA = impulse * j.a1, LB = impulse * j.a2;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    Vec2 Cdot1;
    Cdot1.x = Dot(j.perp, vB - vA) + j.s2 * wB - j.s1 * wA;
    Cdot1.y = wB - wA;
    if (j.enableLimit && j.limitState != 0) {
        const float Cdot2 = Dot(j.u, vB - vA) + j.a2 * wB - j.a1 * wA;
        const float negCdot[3] = {-Cdot1.x, -Cdot1.y, -Cdot2};
        const float f1[3] = {j.impulse[0], j.impulse[1], j.impulse[2]};
        float df[3];
        Solve33(j.mass, negCdot, df);
        j.impulse[0] += df[0]; j.impulse[1] += df[1]; j.impulse[2] += df[2];
        if (j.limitState == 1) j.impulse[2] = Max(j.impulse[2], 0.0f);
        else if (j.limitState == 2) j.impulse[2] = Min(j.impulse[2], 0.0f);
        const Vec2 b = -Cdot1 - (j.impulse[2] - f1[2]) * V(j.mass[6], j.mass[7]);
        const Vec2 f2r = Solve22(j.mass, b) + V(f1[0], f1[1]);
        j.impulse[0] = f2r.x;
        j.impulse[1] = f2r.y;
        df[0] = j.impulse[0] - f1[0]; df[1] = j.impulse[1] - f1[1]; df[2] = j.impulse[2] - f1[2];
        const Vec2 P = df[0] * j.perp + df[2] * j.u;
        const float LA = df[0] * j.s1 + df[1] + df[2] * j.a1;
        const float LB = df[0] * j.s2 + df[1] + df[2] * j.a2;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    } else {
        const Vec2 df = Solve22(j.mass, -Cdot1);
        j.impulse[0] += df.x;
        j.impulse[1] += df.y;
        const Vec2 P = df.x * j.perp;
        const float LA = df.x * j.s1 + df.y;
        const float LB = df.x * j.s2 + df.y;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2PrismaticJoint::SolvePositionConstraints (b2PrismaticJoint.cpp:365-487)
bool PrisSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = cB + rB - cA - rA;
    const Vec2 axis = Mul(qA, j.localXAxisA);
    const float a1 = Cross(d + rA, axis), a2 = Cross(rB, axis);
    const Vec2 perp = Mul(qA, j.localYAxisA);
    const float s1 = Cross(d + rA, perp), s2 = Cross(rB, perp);
    Vec2 C1;
    C1.x = Dot(perp, d);
    C1.y = aB - aA - j.referenceAngle;
    float linearError = Abs(C1.x);
    const float angularError = Abs(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (j.enableLimit) {
        const float translation = Dot(axis, d);
        if (Abs(j.upperAngle - j.lowerAngle) < 2.0f * kLinearSlop) {
            C2 = Clamp(translation, -kMaxLinearCorrection, kMaxLinearCorrection);
            linearError = Max(linearError, Abs(translation));
            active = true;
        } else if (translation <= j.lowerAngle) {
            C2 = Clamp(translation - j.lowerAngle + kLinearSlop, -kMaxLinearCorrection, 0.0f);
            linearError = Max(linearError, j.lowerAngle - translation);
            active = true;
        } else if (translation >= j.upperAngle) {
            C2 = Clamp(translation - j.upperAngle - kLinearSlop, 0.0f, kMaxLinearCorrection);
            linearError = Max(linearError, translation - j.upperAngle);
            active = true;
        }
    }
    float imp[3];
    float K[9];
    K[0] = mA + mB + iA * s1 * s1 + iB * s2 * s2;
    K[1] = iA * s1 + iB * s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    K[4] = k22;
    K[3] = K[1];
    if (active) {
        K[2] = iA * s1 * a1 + iB * s2 * a2;
        K[5] = iA * a1 + iB * a2;
        K[8] = mA + mB + iA * a1 * a1 + iB * a2 * a2;
        K[6] = K[2]; K[7] = K[5];
        const float negC[3] = {-C1.x, -C1.y, -C2};
        Solve33(K, negC, imp);
    } else {
        const Vec2 i2 = Solve22(K, -C1);
        imp[0] = i2.x; imp[1] = i2.y; imp[2] = 0.0f;
    }
    const Vec2 P = imp[0] * perp + imp[2] * axis;
    const float LA = imp[0] * s1 + imp[1] + imp[2] * a1;
    const float LB = imp[0] * s2 + imp[1] + imp[2] * a2;
    cA = cA - mA * P;
    aA -= iA * LA;
    cB = cB + mB * P;
    aB += iB * LB;
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return linearError <= kLinearSlop && angularError <= kAngularSlop;
}


// ---------------------------------------------------------------- wheel joint
// b2WheelJoint::InitVelocityConstraints (Dynamics/Joints/b2WheelJoint.cpp)
void WheelInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = cB + rB - cA - rA;
    j.ay = Mul(qA, j.localYAxisA);
    j.sAy = Cross(d + rA, j.ay);
    j.sBy = Cross(rB, j.ay);
    j.mass[0] = mA + mB + iA * j.sAy * j.sAy + iB * j.sBy * j.sBy;
    if (j.mass[0] > 0.0f) j.mass[0] = 1.0f / j.mass[0];
    j.springMass = 0.0f;
    j.bias = 0.0f;
    j.gamma = 0.0f;
    if (j.frequencyHz > 0.0f) {
        j.ax = Mul(qA, j.localXAxisA);
        j.sAx = Cross(d + rA, j.ax);
        j.sBx = Cross(rB, j.ax);
        const float invMass = mA + mB + iA * j.sAx * j.sAx + iB * j.sBx * j.sBx;
        if (invMass > 0.0f) {
            j.springMass = 1.0f / invMass;
            const float C = Dot(d, j.ax);
            const float omega = 2.0f * kPi * j.frequencyHz;
            const float damp = 2.0f * j.springMass * j.dampingRatio * omega;
            const float k = j.springMass * omega * omega;
            const float h = step.dt;
            j.gamma = h * (damp + h * k);
            if (j.gamma > 0.0f) j.gamma = 1.0f / j.gamma;
            j.bias = C * h * k * j.gamma;
            j.springMass = invMass + j.gamma;
            if (j.springMass > 0.0f) j.springMass = 1.0f / j.springMass;
        }
    } else {
        j.springImpulse = 0.0f;
    }
    if (j.enableMotor) {
        j.motorMass = iA + iB;
        if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    } else {
        j.motorMass = 0.0f;
        j.motorImpulse = 0.0f;
    }
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio;
        j.springImpulse *= step.dtRatio;
        j.motorImpulse *= step.dtRatio;
        const Vec2 P = j.impulse[0] * j.ay + j.springImpulse * j.ax;
        const float LA = j.impulse[0] * j.sAy + j.springImpulse * j.sAx + j.motorImpulse;
        const float LB = j.impulse[0] * j.sBy + j.springImpulse * j.sBx + j.motorImpulse;
        vA = vA - j.invMassA * P;
        wA -= j.invIA * LA;
        vB = vB + j.invMassB * P;
        wB += j.invIB * LB;
    } else {
        j.impulse[0] = 0.0f;
        j.springImpulse = 0.0f;
        j.motorImpulse = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2WheelJoint::SolveVelocityConstraints: spring, rotational motor, point to line
void WheelSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    {
        const float Cdot = Dot(j.ax, vB - vA) + j.sBx * wB - j.sAx * wA;
        const float impulse = -j.springMass * (Cdot + j.bias + j.gamma * j.springImpulse);
        j.springImpulse += impulse;
        const Vec2 P = impulse * j.ax;
        const float LA = impulse * j.sAx, LB = impulse * j.sBx;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    {
        const float Cdot = wB - wA - j.motorSpeed;
        float impulse = -j.motorMass * Cdot;
        const float oldImpulse = j.motorImpulse;
        const float maxImpulse = step.dt * j.maxMotorTorque;
        j.motorImpulse = Clamp(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        const float Cdot = Dot(j.ay, vB - vA) + j.sBy * wB - j.sAy * wA;
        const float impulse = -j.mass[0] * Cdot;
        j.impulse[0] += impulse;
        const Vec2 P = impulse * j.ay;
        const float LA = impulse * j.sAy, LB = impulse * j.sBy;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2WheelJoint::SolvePositionConstraints (its mass uses the velocity step's lever arms m_sAy, m_sBy)
bool WheelSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = (cB - cA) + rB - rA;
    const Vec2 ay = Mul(qA, j.localYAxisA);
    const float sAy = Cross(d + rA, ay), sBy = Cross(rB, ay);
    const float C = Dot(d, ay);
    const float k = j.invMassA + j.invMassB + j.invIA * j.sAy * j.sAy + j.invIB * j.sBy * j.sBy;
    float impulse;
    if (k != 0.0f) impulse = -C / k;
    else impulse = 0.0f;
    const Vec2 P = impulse * ay;
    const float LA = impulse * sAy, LB = impulse * sBy;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * LA;
    cB = cB + j.invMassB * P;
    aB += j.invIB * LB;
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return Abs(C) <= kLinearSlop;
}

// ---------------------------------------------------------------- rope joint
// b2RopeJoint::InitVelocityConstraints (Dynamics/Joints/b2RopeJoint.cpp)
void RopeInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    j.u = cB + j.rB - cA - j.rA;
    j.ropeLength = Length(j.u);
    const float C = j.ropeLength - j.maxLength;
    j.limitState = C > 0.0f ? 2 : 0;
    if (j.ropeLength > kLinearSlop) {
        const float inv = 1.0f / j.ropeLength;
        j.u.x *= inv;
        j.u.y *= inv;
    } else {
        j.u = V(0.0f, 0.0f);
        j.motorMass = 0.0f;
        j.impulse[0] = 0.0f;
        return;
    }
    const float crA = Cross(j.rA, j.u), crB = Cross(j.rB, j.u);
    const float invMass = j.invMassA + j.invIA * crA * crA + j.invMassB + j.invIB * crB * crB;
    j.motorMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio;
        const Vec2 P = j.impulse[0] * j.u;
        vA = vA - j.invMassA * P;
        wA -= j.invIA * Cross(j.rA, P);
        vB = vB + j.invMassB * P;
        wB += j.invIB * Cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

void RopeSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Vec2 vpA = vA + Cross(wA, j.rA);
    const Vec2 vpB = vB + Cross(wB, j.rB);
    const float C = j.ropeLength - j.maxLength;
    float Cdot = Dot(j.u, vpB - vpA);
    if (C < 0.0f) Cdot += step.inv_dt * C;
    float impulse = -j.motorMass * Cdot;
    const float oldImpulse = j.impulse[0];
    j.impulse[0] = Min(0.0f, j.impulse[0] + impulse);
    impulse = j.impulse[0] - oldImpulse;
    const Vec2 P = impulse * j.u;
    vA = vA - j.invMassA * P;
    wA -= j.invIA * Cross(j.rA, P);
    vB = vB + j.invMassB * P;
    wB += j.invIB * Cross(j.rB, P);
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

bool RopeSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    Vec2 u = cB + rB - cA - rA;
    const float length = Normalize(u);
    float C = length - j.maxLength;
    C = Clamp(C, 0.0f, kMaxLinearCorrection);
    const float impulse = -j.motorMass * C;
    const Vec2 P = impulse * u;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * Cross(rA, P);
    cB = cB + j.invMassB * P;
    aB += j.invIB * Cross(rB, P);
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return length - j.maxLength < kLinearSlop;
}

// ---------------------------------------------------------------- friction and motor joints
// b2FrictionJoint (Dynamics/Joints/b2FrictionJoint.cpp) and b2MotorJoint (b2MotorJoint.cpp):
// InitVelocityConstraints; both have no position constraint.
void FrictionMotorInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    const float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    if (j.type == kMotorJoint) {
        j.rA = Mul(qA, -j.localCenterA);
        j.rB = Mul(qB, -j.localCenterB);
    } else {
        j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
        j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    }
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    // b2Mat22 K and its inverse (b2Mat22::GetInverse, Common/b2Math.h)
    const float kexx = mA + mB + iA * j.rA.y * j.rA.y + iB * j.rB.y * j.rB.y;
    const float kexy = -iA * j.rA.x * j.rA.y - iB * j.rB.x * j.rB.y;
    const float keyx = kexy;
    const float keyy = mA + mB + iA * j.rA.x * j.rA.x + iB * j.rB.x * j.rB.x;
    float det = kexx * keyy - keyx * kexy;
    if (det != 0.0f) det = 1.0f / det;
    j.mass[0] = det * keyy; j.mass[2] = -det * keyx;
    j.mass[1] = -det * kexy; j.mass[3] = det * kexx;
    j.motorMass = iA + iB;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    if (j.type == kMotorJoint) {
        const Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
        j.linearError = cB + j.rB - cA - j.rA - Mul(qA, j.linearOffset);
        j.angularError = aB - aA - j.angularOffset;
    }
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio; j.impulse[1] *= step.dtRatio;
        j.impulse[2] *= step.dtRatio;
        const Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = 0.0f;
        j.impulse[2] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// SolveVelocityConstraints of both: angular impulse bounded by dt * maxTorque, linear impulse by
// dt * maxForce in length; the motor joint adds its position errors scaled by inv_dt * correctionFactor
void FrictionMotorSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float h = step.dt;
    const float inv_h = step.inv_dt;
    const bool motor = j.type == kMotorJoint;
    {
        const float Cdot = motor ? wB - wA + inv_h * j.correctionFactor * j.angularError : wB - wA;
        float impulse = -j.motorMass * Cdot;
        const float oldImpulse = j.impulse[2];
        const float maxImpulse = h * j.maxTorque;
        j.impulse[2] = Clamp(j.impulse[2] + impulse, -maxImpulse, maxImpulse);
        impulse = j.impulse[2] - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        Vec2 Cdot = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        if (motor) Cdot = Cdot + inv_h * j.correctionFactor * j.linearError;
        const float* M = j.mass;
        Vec2 impulse = -V(M[0] * Cdot.x + M[2] * Cdot.y, M[1] * Cdot.x + M[3] * Cdot.y);
        const Vec2 oldImpulse = V(j.impulse[0], j.impulse[1]);
        Vec2 li = oldImpulse + impulse;
        const float maxImpulse = h * j.maxForce;
        if (LengthSq(li) > maxImpulse * maxImpulse) {
            Normalize(li);
            li.x *= maxImpulse;
            li.y *= maxImpulse;
        }
        j.impulse[0] = li.x;
        j.impulse[1] = li.y;
        impulse = li - oldImpulse;
        vA = vA - mA * impulse;
        wA -= iA * Cross(j.rA, impulse);
        vB = vB + mB * impulse;
        wB += iB * Cross(j.rB, impulse);
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// ---------------------------------------------------------------- mouse joint
// b2MouseJoint::InitVelocityConstraints (Dynamics/Joints/b2MouseJoint.cpp:95-166): the spring's gamma
// and beta from body B's mass, the 2x2 soft mass, the scaled position error, 2% angular damping of
// body B, warm start.
void MouseInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& B = w->bodies[j.bodyB];
    j.indexB = B.islandIndex;
    j.localCenterB = B.sweep.localCenter;
    j.invMassB = B.invMass;
    j.invIB = B.invI;
    const Vec2 cB = pos[j.indexB].c;
    const Rot qB = RotOf(pos[j.indexB].a);
    Vec2 vB = vel[j.indexB].v;
    float wB = vel[j.indexB].w;
    const float omega = 2.0f * kPi * j.frequencyHz;
    const float dampC = 2.0f * B.mass * j.dampingRatio * omega;
    const float stiff = B.mass * (omega * omega);
    const float h = step.dt;
    j.gamma = h * (dampC + h * stiff);
    if (j.gamma != 0.0f) j.gamma = 1.0f / j.gamma;
    j.beta = h * stiff * j.gamma;
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const float kexx = j.invMassB + j.invIB * j.rB.y * j.rB.y + j.gamma;
    const float kexy = -j.invIB * j.rB.x * j.rB.y;
    const float keyx = kexy;
    const float keyy = j.invMassB + j.invIB * j.rB.x * j.rB.x + j.gamma;
    float det = kexx * keyy - keyx * kexy;
    if (det != 0.0f) det = 1.0f / det;
    j.mass[0] = det * keyy; j.mass[2] = -det * keyx;
    j.mass[1] = -det * kexy; j.mass[3] = det * kexx;
    j.mouseC = cB + j.rB - j.target;
    j.mouseC.x *= j.beta;
    j.mouseC.y *= j.beta;
    wB *= 0.98f;
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio;
        j.impulse[1] *= step.dtRatio;
        const Vec2 P = V(j.impulse[0], j.impulse[1]);
        vB = vB + j.invMassB * P;
        wB += j.invIB * Cross(j.rB, P);
    } else {
        j.impulse[0] = j.impulse[1] = 0.0f;
    }
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2MouseJoint::SolveVelocityConstraints (b2MouseJoint.cpp:168-192): the accumulated impulse is
// rescaled to length dt * maxForce when longer.
void MouseSolveVelocity(Joint& j, const StepInfo& step, Velocity* vel)
{
    Vec2 vB = vel[j.indexB].v;
    float wB = vel[j.indexB].w;
    const Vec2 Cdot = vB + Cross(wB, j.rB);
    const Vec2 old = V(j.impulse[0], j.impulse[1]);
    const Vec2 rhs = -(Cdot + j.mouseC + j.gamma * old);
    const float* M = j.mass;
    const Vec2 d = V(M[0] * rhs.x + M[2] * rhs.y, M[1] * rhs.x + M[3] * rhs.y);
    Vec2 acc = old + d;
    const float maxImpulse = step.dt * j.maxForce;
    if (LengthSq(acc) > maxImpulse * maxImpulse) {
        const float scale = maxImpulse / Length(acc);
        acc.x *= scale;
        acc.y *= scale;
    }
    j.impulse[0] = acc.x;
    j.impulse[1] = acc.y;
    const Vec2 applied = acc - old;
    vB = vB + j.invMassB * applied;
    wB += j.invIB * Cross(j.rB, applied);
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// ---------------------------------------------------------------- pulley joint
// The unit vectors from the ground anchors to the body anchors, zero below 10 linear slops
// (b2PulleyJoint.cpp:99-121 and 218-240).
static void PulleyUnit(Vec2 c, Vec2 r, Vec2 ground, Vec2& u, float& len)
{
    u = c + r - ground;
    len = Length(u);
    if (len > 10.0f * kLinearSlop) {
        const float inv = 1.0f / len;
        u.x *= inv;
        u.y *= inv;
    } else {
        u = V(0.0f, 0.0f);
    }
}

// b2PulleyJoint::InitVelocityConstraints (b2PulleyJoint.cpp:72-154)
void PulleyInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body& A = w->bodies[j.bodyA];
    const Body& B = w->bodies[j.bodyB];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass;
    j.invIA = A.invI; j.invIB = B.invI;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    j.rA = Mul(RotOf(pos[j.indexA].a), j.localAnchorA - j.localCenterA);
    j.rB = Mul(RotOf(pos[j.indexB].a), j.localAnchorB - j.localCenterB);
    float lenA, lenB;
    PulleyUnit(pos[j.indexA].c, j.rA, j.groundAnchorA, j.uA, lenA);
    PulleyUnit(pos[j.indexB].c, j.rB, j.groundAnchorB, j.uB, lenB);
    const float ruA = Cross(j.rA, j.uA), ruB = Cross(j.rB, j.uB);
    const float mA = j.invMassA + j.invIA * ruA * ruA;
    const float mB = j.invMassB + j.invIB * ruB * ruB;
    j.motorMass = mA + j.ratio * j.ratio * mB;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    if (step.warmStarting) {
        j.impulse[0] *= step.dtRatio;
        const Vec2 PA = (-j.impulse[0]) * j.uA;
        const Vec2 PB = (-j.ratio * j.impulse[0]) * j.uB;
        vA = vA + j.invMassA * PA;
        wA += j.invIA * Cross(j.rA, PA);
        vB = vB + j.invMassB * PB;
        wB += j.invIB * Cross(j.rB, PB);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2PulleyJoint::SolveVelocityConstraints (b2PulleyJoint.cpp:156-180)
void PulleySolveVelocity(Joint& j, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w;
    const float Cdot = -Dot(j.uA, vA + Cross(wA, j.rA)) - j.ratio * Dot(j.uB, vB + Cross(wB, j.rB));
    const float impulse = -j.motorMass * Cdot;
    j.impulse[0] += impulse;
    const Vec2 PA = (-impulse) * j.uA;
    const Vec2 PB = (-j.ratio * impulse) * j.uB;
    vA = vA + j.invMassA * PA;
    wA += j.invIA * Cross(j.rA, PA);
    vB = vB + j.invMassB * PB;
    wB += j.invIB * Cross(j.rB, PB);
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
}

// b2PulleyJoint::SolvePositionConstraints (b2PulleyJoint.cpp:182-275): one Newton step on
// constant - lengthA - ratio * lengthB.
bool PulleySolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a;
    const Vec2 rA = Mul(RotOf(aA), j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(RotOf(aB), j.localAnchorB - j.localCenterB);
    Vec2 uA, uB;
    float lenA, lenB;
    PulleyUnit(cA, rA, j.groundAnchorA, uA, lenA);
    PulleyUnit(cB, rB, j.groundAnchorB, uB, lenB);
    const float ruA = Cross(rA, uA), ruB = Cross(rB, uB);
    const float mA = j.invMassA + j.invIA * ruA * ruA;
    const float mB = j.invMassB + j.invIB * ruB * ruB;
    float mass = mA + j.ratio * j.ratio * mB;
    if (mass > 0.0f) mass = 1.0f / mass;
    const float C = j.pulleyConstant - lenA - j.ratio * lenB;
    const float impulse = -mass * C;
    const Vec2 PA = (-impulse) * uA;
    const Vec2 PB = (-j.ratio * impulse) * uB;
    cA = cA + j.invMassA * PA;
    aA += j.invIA * Cross(rA, PA);
    cB = cB + j.invMassB * PB;
    aB += j.invIB * Cross(rB, PB);
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    return Abs(C) < kLinearSlop;
}

// ---------------------------------------------------------------- gear joint
// The gear Jacobian of one coupled joint (b2GearJoint.cpp:171-201, 309-347): for a revolute joint the
// angular terms 1 (scaled by s), for a prismatic joint the axis u in the frame of the joint's body A
// (g) and the lever arms of both bodies; adds the joint's share of the effective mass to *mass, in
// the reference's order (joint 1: mG + mM + ..., joint 2: s*s*(mG + mM) + ...).
static void GearTerms(int type, bool second, float s, Rot qG, Rot qM, Vec2 anchorG, Vec2 anchorM, Vec2 lcG, Vec2 lcM,
                      Vec2 axisG, float mG, float mM, float iG, float iM, Vec2& Jv, float& JwM, float& JwG, Vec2& rM,
                      float* mass)
{
    if (type == kRevoluteJoint) {
        Jv = V(0.0f, 0.0f);
        JwM = s;
        JwG = s;
        *mass += second ? s * s * (iM + iG) : iM + iG;
        return;
    }
    const Vec2 u = Mul(qG, axisG);
    const Vec2 rG = Mul(qG, anchorG - lcG);
    rM = Mul(qM, anchorM - lcM);
    if (second) {
        Jv = s * u;
        JwG = s * Cross(rG, u);
        JwM = s * Cross(rM, u);
        *mass += s * s * (mG + mM) + iG * JwG * JwG + iM * JwM * JwM;
    } else {
        Jv = u;
        JwG = Cross(rG, u);
        JwM = Cross(rM, u);
        *mass += mG + mM + iG * JwG * JwG + iM * JwM * JwM;
    }
}

// b2GearJoint::InitVelocityConstraints (b2GearJoint.cpp:139-240): no dtRatio scaling of the impulse
void GearInit(World* w, Joint& j, const StepInfo& step, Position* pos, Velocity* vel)
{
    const Body &A = w->bodies[j.bodyA], &B = w->bodies[j.bodyB], &Cb = w->bodies[j.bodyC], &Db = w->bodies[j.bodyD];
    j.indexA = A.islandIndex; j.indexB = B.islandIndex; j.indexC = Cb.islandIndex; j.indexD = Db.islandIndex;
    j.localCenterA = A.sweep.localCenter; j.localCenterB = B.sweep.localCenter;
    j.lcC = Cb.sweep.localCenter; j.lcD = Db.sweep.localCenter;
    j.invMassA = A.invMass; j.invMassB = B.invMass; j.invMassC = Cb.invMass; j.invMassD = Db.invMass;
    j.invIA = A.invI; j.invIB = B.invI; j.invIC = Cb.invI; j.invID = Db.invI;
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v, vC = vel[j.indexC].v, vD = vel[j.indexD].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w, wC = vel[j.indexC].w, wD = vel[j.indexD].w;
    const Rot qA = RotOf(pos[j.indexA].a), qB = RotOf(pos[j.indexB].a);
    const Rot qC = RotOf(pos[j.indexC].a), qD = RotOf(pos[j.indexD].a);
    float mass = 0.0f;
    Vec2 rA, rB;
    GearTerms(j.typeA, false, 1.0f, qC, qA, j.localAnchorC, j.localAnchorA, j.lcC, j.localCenterA, j.localAxisC,
              j.invMassC, j.invMassA, j.invIC, j.invIA, j.JvAC, j.JwA, j.JwC, rA, &mass);
    GearTerms(j.typeB, true, j.ratio, qD, qB, j.localAnchorD, j.localAnchorB, j.lcD, j.localCenterB, j.localAxisD,
              j.invMassD, j.invMassB, j.invID, j.invIB, j.JvBD, j.JwB, j.JwD, rB, &mass);
    j.motorMass = mass > 0.0f ? 1.0f / mass : 0.0f;
    if (step.warmStarting) {
        const float P = j.impulse[0];
        vA = vA + (j.invMassA * P) * j.JvAC;
        wA += j.invIA * P * j.JwA;
        vB = vB + (j.invMassB * P) * j.JvBD;
        wB += j.invIB * P * j.JwB;
        vC = vC - (j.invMassC * P) * j.JvAC;
        wC -= j.invIC * P * j.JwC;
        vD = vD - (j.invMassD * P) * j.JvBD;
        wD -= j.invID * P * j.JwD;
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
    vel[j.indexC].v = vC; vel[j.indexC].w = wC;
    vel[j.indexD].v = vD; vel[j.indexD].w = wD;
}

// b2GearJoint::SolveVelocityConstraints (b2GearJoint.cpp:242-277)
void GearSolveVelocity(Joint& j, Velocity* vel)
{
    Vec2 vA = vel[j.indexA].v, vB = vel[j.indexB].v, vC = vel[j.indexC].v, vD = vel[j.indexD].v;
    float wA = vel[j.indexA].w, wB = vel[j.indexB].w, wC = vel[j.indexC].w, wD = vel[j.indexD].w;
    float Cdot = Dot(j.JvAC, vA - vC) + Dot(j.JvBD, vB - vD);
    Cdot += (j.JwA * wA - j.JwC * wC) + (j.JwB * wB - j.JwD * wD);
    const float P = -j.motorMass * Cdot;
    j.impulse[0] += P;
    vA = vA + (j.invMassA * P) * j.JvAC;
    wA += j.invIA * P * j.JwA;
    vB = vB + (j.invMassB * P) * j.JvBD;
    wB += j.invIB * P * j.JwB;
    vC = vC - (j.invMassC * P) * j.JvAC;
    wC -= j.invIC * P * j.JwC;
    vD = vD - (j.invMassD * P) * j.JvBD;
    wD -= j.invID * P * j.JwD;
    vel[j.indexA].v = vA; vel[j.indexA].w = wA;
    vel[j.indexB].v = vB; vel[j.indexB].w = wB;
    vel[j.indexC].v = vC; vel[j.indexC].w = wC;
    vel[j.indexD].v = vD; vel[j.indexD].w = wD;
}

// b2GearJoint::SolvePositionConstraints (b2GearJoint.cpp:279-352): one correction of
// (coordinate1 + ratio * coordinate2) - constant; always reports success
bool GearSolvePosition(Joint& j, Position* pos)
{
    Vec2 cA = pos[j.indexA].c, cB = pos[j.indexB].c, cC = pos[j.indexC].c, cD = pos[j.indexD].c;
    float aA = pos[j.indexA].a, aB = pos[j.indexB].a, aC = pos[j.indexC].a, aD = pos[j.indexD].a;
    const Rot qA = RotOf(aA), qB = RotOf(aB), qC = RotOf(aC), qD = RotOf(aD);
    Vec2 JvAC, JvBD, rA, rB;
    float JwA, JwB, JwC, JwD;
    float mass = 0.0f;
    GearTerms(j.typeA, false, 1.0f, qC, qA, j.localAnchorC, j.localAnchorA, j.lcC, j.localCenterA, j.localAxisC,
              j.invMassC, j.invMassA, j.invIC, j.invIA, JvAC, JwA, JwC, rA, &mass);
    GearTerms(j.typeB, true, j.ratio, qD, qB, j.localAnchorD, j.localAnchorB, j.lcD, j.localCenterB, j.localAxisD,
              j.invMassD, j.invMassB, j.invID, j.invIB, JvBD, JwB, JwD, rB, &mass);
    const float coordA = j.typeA == kRevoluteJoint
                             ? aA - aC - j.referenceAngle
                             : Dot(MulT(qC, rA + (cA - cC)) - (j.localAnchorC - j.lcC), j.localAxisC);
    const float coordB = j.typeB == kRevoluteJoint
                             ? aB - aD - j.referenceAngleB
                             : Dot(MulT(qD, rB + (cB - cD)) - (j.localAnchorD - j.lcD), j.localAxisD);
    const float C = (coordA + j.ratio * coordB) - j.gearConstant;
    float P = 0.0f;
    if (mass > 0.0f) P = -C / mass;
    cA = cA + (j.invMassA * P) * JvAC;
    aA += j.invIA * P * JwA;
    cB = cB + (j.invMassB * P) * JvBD;
    aB += j.invIB * P * JwB;
    cC = cC - (j.invMassC * P) * JvAC;
    aC -= j.invIC * P * JwC;
    cD = cD - (j.invMassD * P) * JvBD;
    aD -= j.invID * P * JwD;
    pos[j.indexA].c = cA; pos[j.indexA].a = aA;
    pos[j.indexB].c = cB; pos[j.indexB].a = aB;
    pos[j.indexC].c = cC; pos[j.indexC].a = aC;
    pos[j.indexD].c = cD; pos[j.indexD].a = aD;
    return true;
}

} // namespace

// ---------------------------------------------------------------- island solve
// b2Island::Solve (Dynamics/b2Island.cpp:185-384)
void World::IslandSolve(const StepInfo& step)
{
    int nb = (int)iBodies.size();
    positions.resize(nb);
    velocities.resize(nb);
    float h = step.dt;
    for (int i = 0; i < nb; ++i) {
        Body& b = bodies[iBodies[i]];
        Vec2 c = b.sweep.c;
        float a = b.sweep.a;
        Vec2 v = b.v;
        float w = b.w;
        b.sweep.c0 = b.sweep.c;
        b.sweep.a0 = b.sweep.a;
        if (b.type == kDynamic) {
            v = v + h * (b.gravityScale * gravity + b.invMass * b.force);
            w += h * b.invI * b.torque;
            v = (1.0f / (1.0f + h * b.linearDamping)) * v;
            w *= 1.0f / (1.0f + h * b.angularDamping);
        }
        positions[i].c = c; positions[i].a = a;
        velocities[i].v = v; velocities[i].w = w;
    }
    ContactSolver cs(this, step, iContacts.data(), (int)iContacts.size(), positions.data(), velocities.data());
    cs.InitVelocity();
    if (step.warmStarting) cs.WarmStart();
    for (int jn : iJoints) {
        Joint& j = joints[jn];
        if (j.type == kDistanceJoint) DistInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kWeldJoint) WeldInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kPrismaticJoint) PrisInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kWheelJoint) WheelInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kRopeJoint) RopeInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kFrictionJoint || j.type == kMotorJoint)
            FrictionMotorInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kMouseJoint) MouseInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kPulleyJoint) PulleyInit(this, j, step, positions.data(), velocities.data());
        else if (j.type == kGearJoint) GearInit(this, j, step, positions.data(), velocities.data());
        else RevInit(this, j, step, positions.data(), velocities.data());
    }
    for (int i = 0; i < step.velocityIterations; ++i) {
        for (int jn : iJoints) {
            Joint& j = joints[jn];
            if (j.type == kDistanceJoint) DistSolveVelocity(j, velocities.data());
            else if (j.type == kWeldJoint) WeldSolveVelocity(j, velocities.data());
            else if (j.type == kPrismaticJoint) PrisSolveVelocity(j, step, velocities.data());
            else if (j.type == kWheelJoint) WheelSolveVelocity(j, step, velocities.data());
            else if (j.type == kRopeJoint) RopeSolveVelocity(j, step, velocities.data());
            else if (j.type == kFrictionJoint || j.type == kMotorJoint)
                FrictionMotorSolveVelocity(j, step, velocities.data());
            else if (j.type == kMouseJoint) MouseSolveVelocity(j, step, velocities.data());
            else if (j.type == kPulleyJoint) PulleySolveVelocity(j, velocities.data());
            else if (j.type == kGearJoint) GearSolveVelocity(j, velocities.data());
            else RevSolveVelocity(j, step, velocities.data());
        }
        cs.SolveVelocity();
    }
    cs.StoreImpulses();
    for (int i = 0; i < nb; ++i) {
        Vec2 c = positions[i].c;
        float a = positions[i].a;
        Vec2 v = velocities[i].v;
        float w = velocities[i].w;
        Vec2 translation = h * v;
        if (Dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = kMaxTranslation / Length(translation);
            v.x *= ratio;
            v.y *= ratio;
        }
        float rotation = h * w;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = kMaxRotation / Abs(rotation);
            w *= ratio;
        }
        c = c + h * v;
        a += h * w;
        positions[i].c = c; positions[i].a = a;
        velocities[i].v = v; velocities[i].w = w;
    }
    bool positionSolved = false;
    for (int i = 0; i < step.positionIterations; ++i) {
        bool contactsOkay = cs.SolvePosition(false, -1, -1);
        bool jointsOkay = true;
        for (int jn : iJoints) {
            Joint& j = joints[jn];
            bool ok = j.type == kDistanceJoint ? DistSolvePosition(j, positions.data())
                      : j.type == kWeldJoint   ? WeldSolvePosition(j, positions.data())
                      : j.type == kPrismaticJoint ? PrisSolvePosition(j, positions.data())
                      : j.type == kWheelJoint ? WheelSolvePosition(j, positions.data())
                      : j.type == kRopeJoint ? RopeSolvePosition(j, positions.data())
                      : j.type == kPulleyJoint ? PulleySolvePosition(j, positions.data())
                      : j.type == kGearJoint ? GearSolvePosition(j, positions.data())
                      : (j.type == kFrictionJoint || j.type == kMotorJoint || j.type == kMouseJoint) ? true
                                               : RevSolvePosition(j, positions.data());
            jointsOkay = jointsOkay && ok;
        }
        if (contactsOkay && jointsOkay) { positionSolved = true; break; }
    }
    for (int i = 0; i < nb; ++i) {
        int bi = iBodies[i];
        Body& b = bodies[bi];
        b.sweep.c = positions[i].c;
        b.sweep.a = positions[i].a;
        b.v = velocities[i].v;
        b.w = velocities[i].w;
        SynchronizeTransform(bi);
    }
    if (recordEvents) {
        for (int i = 0; i < (int)iContacts.size(); ++i) {
            std::vector<float> r = cs.ReportImpulses(i);
            const Contact& c = contacts[iContacts[i]];
            events.push_back(Event{3, c.fA, c.fB, r[0], r[1], r[2], r[3]});
        }
    }
    if (allowSleep) {
        float minSleepTime = kMaxFloat;
        const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
        const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
        for (int i = 0; i < nb; ++i) {
            Body& b = bodies[iBodies[i]];
            if (b.type == kStatic) continue;
            if ((b.flags & kBAutoSleep) == 0 || b.w * b.w > angTolSqr || Dot(b.v, b.v) > linTolSqr) {
                b.sleepTime = 0.0f;
                minSleepTime = 0.0f;
            } else {
                b.sleepTime += h;
                minSleepTime = Min(minSleepTime, b.sleepTime);
            }
        }
        if (minSleepTime >= kTimeToSleep && positionSolved) {
            for (int i = 0; i < nb; ++i) SetAwake(iBodies[i], false);
        }
    }
}

// b2Island::SolveTOI (Dynamics/b2Island.cpp:386-485)
void World::IslandSolveTOI(const StepInfo& sub, int toiA, int toiB)
{
    int nb = (int)iBodies.size();
    positions.resize(nb);
    velocities.resize(nb);
    for (int i = 0; i < nb; ++i) {
        const Body& b = bodies[iBodies[i]];
        positions[i].c = b.sweep.c; positions[i].a = b.sweep.a;
        velocities[i].v = b.v; velocities[i].w = b.w;
    }
    ContactSolver cs(this, sub, iContacts.data(), (int)iContacts.size(), positions.data(), velocities.data());
    for (int i = 0; i < sub.positionIterations; ++i) {
        if (cs.SolvePosition(true, toiA, toiB)) break;
    }
    bodies[iBodies[toiA]].sweep.c0 = positions[toiA].c;
    bodies[iBodies[toiA]].sweep.a0 = positions[toiA].a;
    bodies[iBodies[toiB]].sweep.c0 = positions[toiB].c;
    bodies[iBodies[toiB]].sweep.a0 = positions[toiB].a;
    cs.InitVelocity();
    for (int i = 0; i < sub.velocityIterations; ++i) cs.SolveVelocity();
    float h = sub.dt;
    for (int i = 0; i < nb; ++i) {
        Vec2 c = positions[i].c;
        float a = positions[i].a;
        Vec2 v = velocities[i].v;
        float w = velocities[i].w;
        Vec2 translation = h * v;
        if (Dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = kMaxTranslation / Length(translation);
            v.x *= ratio;
            v.y *= ratio;
        }
        float rotation = h * w;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = kMaxRotation / Abs(rotation);
            w *= ratio;
        }
        c = c + h * v;
        a += h * w;
        positions[i].c = c; positions[i].a = a;
        velocities[i].v = v; velocities[i].w = w;
        int bi = iBodies[i];
        Body& body = bodies[bi];
        body.sweep.c = c;
        body.sweep.a = a;
        body.v = v;
        body.w = w;
        SynchronizeTransform(bi);
    }
    if (recordEvents) {
        for (int i = 0; i < (int)iContacts.size(); ++i) {
            std::vector<float> r = cs.ReportImpulses(i);
            const Contact& c = contacts[iContacts[i]];
            events.push_back(Event{3, c.fA, c.fB, r[0], r[1], r[2], r[3]});
        }
    }
}

// ---------------------------------------------------------------- world step
// b2World::Solve (Dynamics/b2World.cpp:388-577)
void World::Solve(const StepInfo& step)
{
    for (int b = bodyList; b != kNull; b = bodies[b].next) bodies[b].flags &= ~kBIsland;
    for (int c = contactList; c != kNull; c = contacts[c].next) contacts[c].flags &= ~kCIsland;
    for (int j = jointList; j != kNull; j = joints[j].next) joints[j].islandFlag = false;
    stack.resize(bodyCount);
    for (int seed = bodyList; seed != kNull; seed = bodies[seed].next) {
        Body& sb = bodies[seed];
        if (sb.flags & kBIsland) continue;
        if (!sb.IsAwake() || (sb.flags & kBActive) == 0) continue;
        if (sb.type == kStatic) continue;
        iBodies.clear(); iContacts.clear(); iJoints.clear();
        int stackCount = 0;
        stack[stackCount++] = seed;
        sb.flags |= kBIsland;
        while (stackCount > 0) {
            int bi = stack[--stackCount];
            bodies[bi].islandIndex = (int)iBodies.size();
            iBodies.push_back(bi);
            SetAwake(bi, true);
            if (bodies[bi].type == kStatic) continue;
            for (int e = bodies[bi].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1]) {
                int c = e >> 1;
                Contact& ct = contacts[c];
                if (ct.flags & kCIsland) continue;
                if ((ct.flags & kCEnabled) == 0 || (ct.flags & kCTouching) == 0) continue;
                if (fixtures[ct.fA].sensor || fixtures[ct.fB].sensor) continue;
                iContacts.push_back(c);
                ct.flags |= kCIsland;
                int other = EdgeOther(e);
                if (bodies[other].flags & kBIsland) continue;
                stack[stackCount++] = other;
                bodies[other].flags |= kBIsland;
            }
            for (int e = bodies[bi].jointList; e != kNull; e = joints[e >> 1].eNext[e & 1]) {
                Joint& jt = joints[e >> 1];
                if (jt.islandFlag) continue;
                int other = JointEdgeOther(e);
                if ((bodies[other].flags & kBActive) == 0) continue;
                iJoints.push_back(e >> 1);
                jt.islandFlag = true;
                if (bodies[other].flags & kBIsland) continue;
                stack[stackCount++] = other;
                bodies[other].flags |= kBIsland;
            }
        }
        IslandSolve(step);
        for (int bi : iBodies)
            if (bodies[bi].type == kStatic) bodies[bi].flags &= ~kBIsland;
    }
    for (int b = bodyList; b != kNull; b = bodies[b].next) {
        if ((bodies[b].flags & kBIsland) == 0) continue;
        if (bodies[b].type == kStatic) continue;
        SynchronizeFixtures(b);
    }
    FindNewContacts();
}

// b2World::SolveTOI (Dynamics/b2World.cpp:579-896)
void World::SolveTOI(const StepInfo& step)
{
    if (stepComplete) {
        for (int b = bodyList; b != kNull; b = bodies[b].next) {
            bodies[b].flags &= ~kBIsland;
            bodies[b].sweep.alpha0 = 0.0f;
        }
        for (int c = contactList; c != kNull; c = contacts[c].next) {
            contacts[c].flags &= ~(kCToi | kCIsland);
            contacts[c].toiCount = 0;
            contacts[c].toi = 1.0f;
        }
    }
    for (;;) {
        int minContact = kNull;
        float minAlpha = 1.0f;
        for (int c = contactList; c != kNull; c = contacts[c].next) {
            Contact& ct = contacts[c];
            if ((ct.flags & kCEnabled) == 0) continue;
            if (ct.toiCount > kMaxSubSteps) continue;
            float alpha = 1.0f;
            if (ct.flags & kCToi) {
                alpha = ct.toi;
            } else {
                const Fixture& fA = fixtures[ct.fA];
                const Fixture& fB = fixtures[ct.fB];
                if (fA.sensor || fB.sensor) continue;
                Body& bA = bodies[fA.body];
                Body& bB = bodies[fB.body];
                bool activeA = bA.IsAwake() && bA.type != kStatic;
                bool activeB = bB.IsAwake() && bB.type != kStatic;
                if (!activeA && !activeB) continue;
                bool collideA = (bA.flags & kBBullet) != 0 || bA.type != kDynamic;
                bool collideB = (bB.flags & kBBullet) != 0 || bB.type != kDynamic;
                if (!collideA && !collideB) continue;
                float alpha0 = bA.sweep.alpha0;
                if (bA.sweep.alpha0 < bB.sweep.alpha0) {
                    alpha0 = bB.sweep.alpha0;
                    SweepAdvance(bA.sweep, alpha0);
                } else if (bB.sweep.alpha0 < bA.sweep.alpha0) {
                    alpha0 = bA.sweep.alpha0;
                    SweepAdvance(bB.sweep, alpha0);
                }
                DistanceProxy pa, pb;
                ProxyOf(&pa, fA.shape);
                ProxyOf(&pb, fB.shape);
                int state;
                float beta;
                TimeOfImpact(&state, &beta, pa, pb, bA.sweep, bB.sweep, 1.0f);
                if (state == kToiTouching) alpha = Min(alpha0 + (1.0f - alpha0) * beta, 1.0f);
                else alpha = 1.0f;
                ct.toi = alpha;
                ct.flags |= kCToi;
            }
            if (alpha < minAlpha) { minContact = c; minAlpha = alpha; }
        }
        if (minContact == kNull || 1.0f - 10.0f * kEpsilon < minAlpha) {
            stepComplete = true;
            break;
        }
        int bA = fixtures[contacts[minContact].fA].body, bB = fixtures[contacts[minContact].fB].body;
        Sweep backup1 = bodies[bA].sweep, backup2 = bodies[bB].sweep;
        Advance(bA, minAlpha);
        Advance(bB, minAlpha);
        Update(minContact);
        contacts[minContact].flags &= ~kCToi;
        ++contacts[minContact].toiCount;
        if ((contacts[minContact].flags & kCEnabled) == 0 || (contacts[minContact].flags & kCTouching) == 0) {
            contacts[minContact].flags &= ~kCEnabled;
            bodies[bA].sweep = backup1;
            bodies[bB].sweep = backup2;
            SynchronizeTransform(bA);
            SynchronizeTransform(bB);
            continue;
        }
        SetAwake(bA, true);
        SetAwake(bB, true);
        iBodies.clear(); iContacts.clear(); iJoints.clear();
        const int bodyCap = 2 * kMaxTOIContacts, contactCap = kMaxTOIContacts;
        bodies[bA].islandIndex = 0; iBodies.push_back(bA);
        bodies[bB].islandIndex = 1; iBodies.push_back(bB);
        iContacts.push_back(minContact);
        bodies[bA].flags |= kBIsland;
        bodies[bB].flags |= kBIsland;
        contacts[minContact].flags |= kCIsland;
        int pair[2] = {bA, bB};
        for (int k = 0; k < 2; ++k) {
            int body = pair[k];
            if (bodies[body].type != kDynamic) continue;
            for (int e = bodies[body].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1]) {
                if ((int)iBodies.size() == bodyCap) break;
                if ((int)iContacts.size() == contactCap) break;
                int c = e >> 1;
                Contact& ct = contacts[c];
                if (ct.flags & kCIsland) continue;
                int other = EdgeOther(e);
                if (bodies[other].type == kDynamic && (bodies[body].flags & kBBullet) == 0 && (bodies[other].flags & kBBullet) == 0)
                    continue;
                if (fixtures[ct.fA].sensor || fixtures[ct.fB].sensor) continue;
                Sweep backup = bodies[other].sweep;
                if ((bodies[other].flags & kBIsland) == 0) Advance(other, minAlpha);
                Update(c);
                if ((contacts[c].flags & kCEnabled) == 0 || (contacts[c].flags & kCTouching) == 0) {
                    bodies[other].sweep = backup;
                    SynchronizeTransform(other);
                    continue;
                }
                contacts[c].flags |= kCIsland;
                iContacts.push_back(c);
                if (bodies[other].flags & kBIsland) continue;
                bodies[other].flags |= kBIsland;
                if (bodies[other].type != kStatic) SetAwake(other, true);
                bodies[other].islandIndex = (int)iBodies.size();
                iBodies.push_back(other);
            }
        }
        StepInfo sub;
        sub.dt = (1.0f - minAlpha) * step.dt;
        sub.inv_dt = 1.0f / sub.dt;
        sub.dtRatio = 1.0f;
        sub.positionIterations = 20;
        sub.velocityIterations = step.velocityIterations;
        sub.warmStarting = false;
        IslandSolveTOI(sub, bodies[bA].islandIndex, bodies[bB].islandIndex);
        for (int bi : iBodies) {
            bodies[bi].flags &= ~kBIsland;
            if (bodies[bi].type != kDynamic) continue;
            SynchronizeFixtures(bi);
            for (int e = bodies[bi].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1])
                contacts[e >> 1].flags &= ~(kCToi | kCIsland);
        }
        FindNewContacts();
        if (subStepping) { stepComplete = false; break; }
    }
}

// b2World::Step (Dynamics/b2World.cpp:899-963)
void World::Step(float dt, int vi, int pi)
{
    stepPairs.clear();
    events.clear();
    if (wflags & 0x1) {
        FindNewContacts();
        wflags &= ~0x1u;
    }
    wflags |= 0x2;
    StepInfo step;
    step.dt = dt;
    step.velocityIterations = vi;
    step.positionIterations = pi;
    step.inv_dt = dt > 0.0f ? 1.0f / dt : 0.0f;
    step.dtRatio = inv_dt0 * dt;
    step.warmStarting = warmStarting;
    Collide();
    if (stepComplete && step.dt > 0.0f) Solve(step);
    if (continuous && step.dt > 0.0f) SolveTOI(step);
    if (step.dt > 0.0f) inv_dt0 = step.inv_dt;
    if (wflags & 0x4) {
        for (int b = bodyList; b != kNull; b = bodies[b].next) {
            bodies[b].force = V(0.0f, 0.0f);
            bodies[b].torque = 0.0f;
        }
    }
    wflags &= ~0x2u;
}

} // namespace b2o

// ---------------------------------------------------------------- destruction
namespace b2o {

// b2World::DestroyJoint (Dynamics/b2World.cpp:274-362)
void World::DestroyJoint(int jn)
{
    Joint& j = joints[jn];
    const bool collideConnected = j.collideConnected;
    if (j.prev != kNull) joints[j.prev].next = j.next;
    if (j.next != kNull) joints[j.next].prev = j.prev;
    if (jn == jointList) jointList = j.next;
    const int bA = j.bodyA, bB = j.bodyB;
    SetAwake(bA, true);
    SetAwake(bB, true);
    for (int side = 0; side < 2; ++side) {
        const int body = side == 0 ? bA : bB;
        const int e = 2 * jn + side;
        const int pe = j.ePrev[side], ne = j.eNext[side];
        if (pe != kNull) joints[pe >> 1].eNext[pe & 1] = ne;
        if (ne != kNull) joints[ne >> 1].ePrev[ne & 1] = pe;
        if (bodies[body].jointList == e) bodies[body].jointList = ne;
        j.ePrev[side] = j.eNext[side] = kNull;
    }
    --jointCount;
    if (!collideConnected)
        for (int e = bodies[bB].contactList; e != kNull; e = contacts[e >> 1].eNext[e & 1])
            if (EdgeOther(e) == bA) contacts[e >> 1].flags |= kCFilter;
}

// b2World::DestroyBody (Dynamics/b2World.cpp:133-212): attached joints (each announced to the
// destruction listener first), attached contacts, fixtures with their proxies (each announced), then
// the body leaves the body list.
void World::DestroyBody(int bi)
{
    goodbyes.clear();
    for (int e = bodies[bi].jointList; e != kNull;) {
        const int jn = e >> 1;
        e = joints[jn].eNext[e & 1];
        goodbyes.push_back({0, jn});
        DestroyJoint(jn);
        bodies[bi].jointList = e;
    }
    bodies[bi].jointList = kNull;
    for (int e = bodies[bi].contactList; e != kNull;) {
        const int c = e >> 1;
        e = contacts[c].eNext[e & 1];
        Destroy(c);
    }
    bodies[bi].contactList = kNull;
    for (int f = bodies[bi].fixtureList; f != kNull;) {
        Fixture& fx = fixtures[f];
        const int next = fx.next;
        // a chain is one b2Fixture: announced once, at its first child
        if (fx.shape.chain != 2) goodbyes.push_back({1, f});
        if (fx.proxyCount > 0) {
            bp.DestroyProxy(fx.proxyId);
            fx.proxyId = kNull;
            fx.proxyCount = 0;
        }
        fx.body = kNull;
        fx.next = kNull;
        bodies[bi].fixtureList = next;
        f = next;
    }
    Body& b = bodies[bi];
    if (b.prev != kNull) bodies[b.prev].next = b.next;
    if (b.next != kNull) bodies[b.next].prev = b.prev;
    if (bi == bodyList) bodyList = b.next;
    --bodyCount;
    b = Body();
    b.alive = false;
}

// b2Body::DestroyFixture (Dynamics/b2Body.cpp:216-281): the fixture leaves the body's list, its
// contacts are destroyed in the body's contact-list order, its proxies are destroyed and the body's
// mass data is reset. A chain (its first child's index) goes with all of its children.
void World::DestroyFixture(int f)
{
    goodbyes.clear();
    const int bi = fixtures[f].body;
    int last = f;
    if (fixtures[f].shape.chain == 1)
        while (last + 1 < (int)fixtures.size() && fixtures[last + 1].body == bi && fixtures[last + 1].shape.chain == 2)
            ++last;
    auto mine = [&](int id) { return id >= f && id <= last; };
    // unlink the children (consecutive in the list) from the body's fixture list
    int* node = &bodies[bi].fixtureList;
    while (*node != kNull && !mine(*node)) node = &fixtures[*node].next;
    int after = *node;
    while (after != kNull && mine(after)) after = fixtures[after].next;
    if (*node != kNull) *node = after;
    for (int e = bodies[bi].contactList; e != kNull;) {
        const int c = e >> 1;
        e = contacts[c].eNext[e & 1];
        if (mine(contacts[c].fA) || mine(contacts[c].fB)) Destroy(c);
    }
    for (int id = f; id <= last; ++id) {
        Fixture& fx = fixtures[id];
        if ((bodies[bi].flags & kBActive) && fx.proxyCount > 0) {
            bp.DestroyProxy(fx.proxyId);
        }
        fx.proxyId = kNull;
        fx.proxyCount = 0;
        fx.body = kNull;
        fx.next = kNull;
    }
    ResetMassData(bi);
}

} // namespace b2o

namespace b2o {

// default b2ContactFilter::ShouldCollide (Dynamics/b2WorldCallbacks.cpp:26-38)
bool World::DefaultFilter(int fA, int fB) const
{
    const Fixture& fa = fixtures[fA];
    const Fixture& fb = fixtures[fB];
    if (fa.group == fb.group && fa.group != 0) return fa.group > 0;
    return (fa.mask & fb.category) != 0 && (fa.category & fb.mask) != 0;
}

// The world's b2ContactFilter: the default, or the test filter (the first filterStatic fixtures keep
// the default; any other pair collides unless (fixtureA + fixtureB) % filterModulus == 0)
bool World::FilterShouldCollide(int fA, int fB) const
{
    if (filterModulus <= 0 || fA < filterStatic || fB < filterStatic) return DefaultFilter(fA, fB);
    return (fA + fB) % filterModulus != 0;
}

} // namespace b2o
