// Oracle (test infrastructure only): a C-ABI driver around the UNMODIFIED reference Box2D 2.3.2
// (namespace box2dref, Regression/box2d-ref/Box2DRef in the reference tree), compiled from the
// reference sources in place by oracle/Makefile into oracle/_ref/. It builds scenes through the
// reference's own public API (b2World::CreateBody, b2Body::CreateFixture, b2World::CreateJoint,
// b2World::Step) and reads state back for golden-vector generation. Nothing here is product code.
//
// Private members are read (not written) for the dump: fat AABBs, proxy ids, contact flags.
#include <algorithm>
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>
#define private public
#define protected public
#include <Box2DRef/Box2D.h>
#undef private
#undef protected

using namespace box2dref;

namespace {

int fixture_index(const b2Fixture* f) { return (int)(intptr_t)f->GetUserData() - 1; }
int body_index(const b2Body* b) { return (int)(intptr_t)b->GetUserData() - 1; }

struct RefWorld;

// b2DestructionListener recording its calls as {0 joint / 1 fixture, creation index}
struct Goodbye : public b2DestructionListener {
    RefWorld* owner = nullptr;
    std::vector<int> calls;
    void SayGoodbye(b2Joint* joint) override;
    void SayGoodbye(b2Fixture* fixture) override;
};

// A b2ContactListener whose PreSolve applies a rule per fixture pair (bits per fixture: 1 ghost,
// 2 ice, 4 bouncy; a contact between two fixtures sharing a bit is disabled, gets friction 0 or
// restitution 0.9).
struct PreSolveRule : public b2ContactListener {
    std::vector<int> bits;
    void PreSolve(b2Contact* contact, const b2Manifold*) override
    {
        const int a = fixture_index(contact->GetFixtureA()) + contact->GetChildIndexA();
        const int b = fixture_index(contact->GetFixtureB()) + contact->GetChildIndexB();
        const int both = (a < (int)bits.size() ? bits[a] : 0) & (b < (int)bits.size() ? bits[b] : 0);
        if (both & 1) contact->SetEnabled(false);
        if (both & 2) contact->SetFriction(0.0f);
        if (both & 4) contact->SetRestitution(0.9f);
    }
};

// A b2ContactFilter for tests: fixtures below firstOther keep the default filter; any other pair
// collides unless (fixtureA + fixtureB) % modulus == 0.
struct FilterRule : public b2ContactFilter {
    int modulus = 0, firstOther = 0;
    bool ShouldCollide(b2Fixture* a, b2Fixture* b) override
    {
        const int fa = fixture_index(a), fb = fixture_index(b);
        if (fa < firstOther || fb < firstOther) return b2ContactFilter::ShouldCollide(a, b);
        return (fa + fb) % modulus != 0;
    }
};

struct RefWorld {
    b2World world;
    PreSolveRule rule;
    FilterRule filter;
    std::vector<b2Body*> bodies;      // creation order; null once destroyed
    std::vector<b2Fixture*> fixtures; // creation order (a chain's children share one); null once destroyed
    std::vector<b2Joint*> joints;     // creation order; null once destroyed
    Goodbye goodbye;
    explicit RefWorld(const b2Vec2& g) : world(g)
    {
        goodbye.owner = this;
        world.SetDestructionListener(&goodbye);
    }
};

void Goodbye::SayGoodbye(b2Joint* joint)
{
    for (size_t i = 0; i < owner->joints.size(); ++i)
        if (owner->joints[i] == joint) { calls.push_back(0); calls.push_back((int)i); }
}
void Goodbye::SayGoodbye(b2Fixture* fixture)
{
    calls.push_back(1);
    calls.push_back((int)(intptr_t)fixture->GetUserData() - 1);
}


} // namespace

extern "C" {

void* rw_create(float gx, float gy) { return new RefWorld(b2Vec2(gx, gy)); }
void rw_destroy(void* h) { delete static_cast<RefWorld*>(h); }

void rw_config(void* h, int allowSleep, int warmStarting, int continuous, int subStepping)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->world.SetAllowSleeping(allowSleep != 0);
    w->world.SetWarmStarting(warmStarting != 0);
    w->world.SetContinuousPhysics(continuous != 0);
    w->world.SetSubStepping(subStepping != 0);
}

// f = {x, y, angle, vx, vy, w, linearDamping, angularDamping, gravityScale}
// flags: 1 allowSleep, 2 awake, 4 fixedRotation, 8 bullet, 16 active
int rw_body(void* h, int type, const float* f, int flags)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    b2BodyDef bd;
    bd.type = (b2BodyType)type;
    bd.position.Set(f[0], f[1]);
    bd.angle = f[2];
    bd.linearVelocity.Set(f[3], f[4]);
    bd.angularVelocity = f[5];
    bd.linearDamping = f[6];
    bd.angularDamping = f[7];
    bd.gravityScale = f[8];
    bd.allowSleep = (flags & 1) != 0;
    bd.awake = (flags & 2) != 0;
    bd.fixedRotation = (flags & 4) != 0;
    bd.bullet = (flags & 8) != 0;
    bd.active = (flags & 16) != 0;
    bd.userData = (void*)(intptr_t)(w->bodies.size() + 1);
    b2Body* b = w->world.CreateBody(&bd);
    w->bodies.push_back(b);
    return (int)w->bodies.size() - 1;
}

// shapeType 0 circle: s = {px, py, radius}
// shapeType 1 edge:   s = {v1x, v1y, v2x, v2y, v0x, v0y, v3x, v3y, hasV0, hasV3}
// shapeType 2 polygon from points: s = n points (b2PolygonShape::Set)
// shapeType 3 box:    s = {hx, hy} (SetAsBox(hx, hy)) or {hx, hy, cx, cy, angle} when n == 5
// mat = {density, friction, restitution}; filt = {categoryBits, maskBits, groupIndex, isSensor}
int rw_fixture(void* h, int body, int shapeType, const float* s, int n, const float* mat, const int* filt)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    b2FixtureDef fd;
    b2CircleShape circle;
    b2EdgeShape edge;
    b2PolygonShape poly;
    switch (shapeType) {
    case 0:
        circle.m_p.Set(s[0], s[1]);
        circle.m_radius = s[2];
        fd.shape = &circle;
        break;
    case 1:
        if (s[10] != 0.0f) return -1;  // chain children are built by rw_build (rw_chain)
        edge.Set(b2Vec2(s[0], s[1]), b2Vec2(s[2], s[3]));
        edge.m_vertex0.Set(s[4], s[5]);
        edge.m_vertex3.Set(s[6], s[7]);
        edge.m_hasVertex0 = s[8] != 0.0f;
        edge.m_hasVertex3 = s[9] != 0.0f;
        fd.shape = &edge;
        break;
    case 2: {
        b2Vec2 pts[b2_maxPolygonVertices];
        for (int i = 0; i < n && i < b2_maxPolygonVertices; ++i) pts[i].Set(s[2 * i], s[2 * i + 1]);
        poly.Set(pts, n);
        fd.shape = &poly;
        break;
    }
    case 3:
        if (n == 5) poly.SetAsBox(s[0], s[1], b2Vec2(s[2], s[3]), s[4]);
        else poly.SetAsBox(s[0], s[1]);
        fd.shape = &poly;
        break;
    default:
        return -1;
    }
    fd.density = mat[0];
    fd.friction = mat[1];
    fd.restitution = mat[2];
    fd.filter.categoryBits = (uint16)filt[0];
    fd.filter.maskBits = (uint16)filt[1];
    fd.filter.groupIndex = (int16)filt[2];
    fd.isSensor = filt[3] != 0;
    fd.userData = (void*)(intptr_t)(w->fixtures.size() + 1);
    b2Fixture* fx = w->bodies[body]->CreateFixture(&fd);
    w->fixtures.push_back(fx);
    return (int)w->fixtures.size() - 1;
}

// f = {localAnchorA.x, .y, localAnchorB.x, .y, referenceAngle, lowerAngle, upperAngle, motorSpeed, maxMotorTorque}
// flags: 1 enableLimit, 2 enableMotor, 4 collideConnected
int rw_revolute(void* h, int bodyA, int bodyB, const float* f, int flags)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    b2RevoluteJointDef jd;
    jd.bodyA = w->bodies[bodyA];
    jd.bodyB = w->bodies[bodyB];
    jd.localAnchorA.Set(f[0], f[1]);
    jd.localAnchorB.Set(f[2], f[3]);
    jd.referenceAngle = f[4];
    jd.lowerAngle = f[5];
    jd.upperAngle = f[6];
    jd.motorSpeed = f[7];
    jd.maxMotorTorque = f[8];
    jd.enableLimit = (flags & 1) != 0;
    jd.enableMotor = (flags & 2) != 0;
    jd.collideConnected = (flags & 4) != 0;
    w->joints.push_back(w->world.CreateJoint(&jd));
    return (int)w->joints.size() - 1;
}

// b2World::CreateJoint with a distance (type 1) or weld (type 2) definition; f as gb_create_joints.
int rw_joint(void* h, int type, int bodyA, int bodyB, const float* f, int flags)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    if (type == 0) return rw_revolute(h, bodyA, bodyB, f, flags);
    if (type == 1) {
        b2DistanceJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.length = f[4];
        jd.frequencyHz = f[5];
        jd.dampingRatio = f[6];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 2) {
        b2WeldJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.referenceAngle = f[4];
        jd.frequencyHz = f[5];
        jd.dampingRatio = f[6];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 4) {
        b2WheelJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.localAxisA.Set(f[4], f[5]);
        jd.maxMotorTorque = f[6];
        jd.motorSpeed = f[7];
        jd.frequencyHz = f[8];
        jd.dampingRatio = f[9];
        jd.enableMotor = (flags & 2) != 0;
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 5) {
        b2RopeJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.maxLength = f[4];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 6) {
        b2FrictionJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.maxForce = f[4];
        jd.maxTorque = f[5];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 7) {
        b2MotorJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.linearOffset.Set(f[0], f[1]);
        jd.angularOffset = f[2];
        jd.maxForce = f[3];
        jd.maxTorque = f[4];
        jd.correctionFactor = f[5];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 8) {
        b2MouseJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.target.Set(f[0], f[1]);
        jd.maxForce = f[2];
        jd.frequencyHz = f[3];
        jd.dampingRatio = f[4];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 10) {
        b2GearJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.joint1 = w->joints[(int)f[0]];
        jd.joint2 = w->joints[(int)f[1]];
        jd.ratio = f[2];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else if (type == 9) {
        b2PulleyJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.groundAnchorA.Set(f[0], f[1]);
        jd.groundAnchorB.Set(f[2], f[3]);
        jd.localAnchorA.Set(f[4], f[5]);
        jd.localAnchorB.Set(f[6], f[7]);
        jd.lengthA = f[8];
        jd.lengthB = f[9];
        jd.ratio = f[10];
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    } else {
        b2PrismaticJointDef jd;
        jd.bodyA = w->bodies[bodyA];
        jd.bodyB = w->bodies[bodyB];
        jd.localAnchorA.Set(f[0], f[1]);
        jd.localAnchorB.Set(f[2], f[3]);
        jd.localAxisA.Set(f[4], f[5]);
        jd.referenceAngle = f[6];
        jd.lowerTranslation = f[7];
        jd.upperTranslation = f[8];
        jd.maxMotorForce = f[9];
        jd.motorSpeed = f[10];
        jd.enableLimit = (flags & 1) != 0;
        jd.enableMotor = (flags & 2) != 0;
        jd.collideConnected = (flags & 4) != 0;
        w->joints.push_back(w->world.CreateJoint(&jd));
    }
    return (int)w->joints.size() - 1;
}

int rw_chain(void* h, int body, int nchild, const float* s, const float* mat, const int* filt);

// Bulk scene build: body b is created, then its fixtures (fbody is non-decreasing), then all joints.
void rw_build(void* h, int nb, const int* btype, const float* bf, const int* bflags, int nf, const int* fbody,
              const int* ftype, const float* fshape, const int* fn, const float* fmat, const int* ffilt, int nj,
              const int* ja, const int* jb, const float* jf, const int* jflags)
{
    int fi = 0;
    for (int b = 0; b < nb; ++b) {
        rw_body(h, btype[b], bf + 9 * b, bflags[b]);
        while (fi < nf && fbody[fi] == b) {
            const float* s = fshape + 16 * fi;
            if (ftype[fi] == 1 && s[10] == 1.0f) {
                int n = 1;
                while (fi + n < nf && fbody[fi + n] == b && ftype[fi + n] == 1 && fshape[16 * (fi + n) + 10] == 2.0f) ++n;
                rw_chain(h, b, n, s, fmat + 3 * fi, ffilt + 4 * fi);
                fi += n;
                continue;
            }
            rw_fixture(h, b, ftype[fi], s, fn[fi], fmat + 3 * fi, ffilt + 4 * fi);
            ++fi;
        }
    }
    for (int j = 0; j < nj; ++j) rw_revolute(h, ja[j], jb[j], jf + 12 * j, jflags[j]);
}

void rw_step(void* h, float dt, int vi, int pi) { static_cast<RefWorld*>(h)->world.Step(dt, vi, pi); }

// A b2Body state change between steps through the reference's own methods. op: the C-ABI's GB_EDIT_*.
void rw_body_edit(void* h, int op, int body, int wake, const float* v)
{
    if (op == 9) { // body is the joint index of a mouse joint
        static_cast<b2MouseJoint*>(static_cast<RefWorld*>(h)->joints[body])->SetTarget(b2Vec2(v[0], v[1]));
        return;
    }
    b2Body* b = static_cast<RefWorld*>(h)->bodies[body];
    const bool w = wake != 0;
    switch (op) {
    case 0: b->SetTransform(b2Vec2(v[0], v[1]), v[2]); break;
    case 1: b->SetLinearVelocity(b2Vec2(v[0], v[1])); break;
    case 2: b->SetAngularVelocity(v[0]); break;
    case 3: b->SetAwake(v[0] != 0.0f); break;
    case 4: b->ApplyForce(b2Vec2(v[0], v[1]), b2Vec2(v[2], v[3]), w); break;
    case 5: b->ApplyForceToCenter(b2Vec2(v[0], v[1]), w); break;
    case 6: b->ApplyTorque(v[0], w); break;
    case 7: b->ApplyLinearImpulse(b2Vec2(v[0], v[1]), b2Vec2(v[2], v[3]), w); break;
    case 8: b->ApplyAngularImpulse(v[0], w); break;
    default: break;
    }
}

int rw_body_count(void* h) { return (int)static_cast<RefWorld*>(h)->bodies.size(); }

// Forget every pointer a destruction made dangling: joints and fixtures that are no longer attached
// to a live body, after a DestroyBody / DestroyJoint / DestroyFixture call.
static void ForgetDestroyed(RefWorld* w, b2Body* gone)
{
    for (size_t i = 0; i < w->bodies.size(); ++i)
        if (w->bodies[i] == gone) w->bodies[i] = nullptr;
    std::vector<b2Joint*> live;
    for (b2Joint* j = w->world.GetJointList(); j; j = j->GetNext()) live.push_back(j);
    for (b2Joint*& j : w->joints)
        if (j && std::find(live.begin(), live.end(), j) == live.end()) j = nullptr;
    std::vector<b2Fixture*> liveF;
    for (b2Body* b = w->world.GetBodyList(); b; b = b->GetNext())
        for (b2Fixture* f = b->GetFixtureList(); f; f = f->GetNext()) liveF.push_back(f);
    for (b2Fixture*& f : w->fixtures)
        if (f && std::find(liveF.begin(), liveF.end(), f) == liveF.end()) f = nullptr;
}
static int TakeGoodbyes(RefWorld* w, int* calls, int cap)
{
    const int n = (int)w->goodbye.calls.size() / 2;
    for (int i = 0; i < 2 * n && i < 2 * cap; ++i) calls[i] = w->goodbye.calls[i];
    w->goodbye.calls.clear();
    return n;
}
void rw_set_filter_rule(void* h, int modulus, int firstOther)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->filter.modulus = modulus;
    w->filter.firstOther = firstOther;
    w->world.SetContactFilter(&w->filter);
}
void rw_set_settings(void* h, float gx, float gy, int allowSleep, int warm, int continuous, int subStepping,
                     int autoClear)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->world.SetGravity(b2Vec2(gx, gy));
    w->world.SetAllowSleeping(allowSleep != 0);
    w->world.SetWarmStarting(warm != 0);
    w->world.SetContinuousPhysics(continuous != 0);
    w->world.SetSubStepping(subStepping != 0);
    w->world.SetAutoClearForces(autoClear != 0);
}
// b2Body property changes between steps (prop: the C-ABI's GB_BODY_* code)
void rw_body_set(void* h, int b, int prop, const float* v)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    b2Body* body = w->bodies[b];
    const bool flag = v[0] != 0.0f;
    switch (prop) {
    case 0: body->SetType((b2BodyType)(int)v[0]); break;
    case 1: body->SetActive(flag); break;
    case 2: body->SetFixedRotation(flag); break;
    case 3: body->SetBullet(flag); break;
    case 4: body->SetSleepingAllowed(flag); break;
    case 5: body->SetLinearDamping(v[0]); break;
    case 6: body->SetAngularDamping(v[0]); break;
    case 7: body->SetGravityScale(v[0]); break;
    case 8: {
        b2MassData md;
        md.mass = v[0];
        md.center.Set(v[1], v[2]);
        md.I = v[3];
        body->SetMassData(&md);
        break;
    }
    case 9: body->ResetMassData(); break;
    default: break;
    }
}
// b2PolygonShape::Set (mode 0), SetAsBox(hx, hy) (mode 1), SetAsBox(hx, hy, center, angle) (mode 2):
// out = centroid, 8 vertices, 8 normals; returns the vertex count
int rw_polygon_shape(int mode, const float* in, int n, float* out)
{
    b2PolygonShape s;
    if (mode == 0) {
        b2Vec2 pts[b2_maxPolygonVertices];
        for (int i = 0; i < n; ++i) pts[i].Set(in[2 * i], in[2 * i + 1]);
        s.Set(pts, n);
    } else if (mode == 1) {
        s.SetAsBox(in[0], in[1]);
    } else {
        s.SetAsBox(in[0], in[1], b2Vec2(in[2], in[3]), in[4]);
    }
    out[0] = s.m_centroid.x;
    out[1] = s.m_centroid.y;
    for (int i = 0; i < b2_maxPolygonVertices; ++i) {
        out[2 + 2 * i] = i < s.m_count ? s.m_vertices[i].x : 0.0f;
        out[3 + 2 * i] = i < s.m_count ? s.m_vertices[i].y : 0.0f;
        out[18 + 2 * i] = i < s.m_count ? s.m_normals[i].x : 0.0f;
        out[19 + 2 * i] = i < s.m_count ? s.m_normals[i].y : 0.0f;
    }
    return s.m_count;
}
// b2Fixture::TestPoint (op 0: in = point; out[0] 1 inside), RayCast (op 1: in = p1, p2, maxFraction;
// out = hit, normal, fraction) and GetAABB (op 2: out = lower, upper) of a fixture's first child
void rw_fixture_query(void* h, int f, int op, const float* in, float* out)
{
    const b2Fixture* fx = static_cast<RefWorld*>(h)->fixtures[f];
    if (op == 0) {
        out[0] = fx->TestPoint(b2Vec2(in[0], in[1])) ? 1.0f : 0.0f;
    } else if (op == 1) {
        b2RayCastInput input;
        input.p1.Set(in[0], in[1]);
        input.p2.Set(in[2], in[3]);
        input.maxFraction = in[4];
        b2RayCastOutput output;
        output.normal.SetZero();
        output.fraction = 0.0f;
        const bool hit = fx->RayCast(&output, input, 0);
        out[0] = hit ? 1.0f : 0.0f;
        out[1] = hit ? output.normal.x : 0.0f;
        out[2] = hit ? output.normal.y : 0.0f;
        out[3] = hit ? output.fraction : 0.0f;
    } else if (op == 3) {
        b2MassData md;
        fx->GetMassData(&md);
        out[0] = md.mass;
        out[1] = md.center.x;
        out[2] = md.center.y;
        out[3] = md.I;
    } else {
        const b2AABB& a = fx->GetAABB(0);
        out[0] = a.lowerBound.x;
        out[1] = a.lowerBound.y;
        out[2] = a.upperBound.x;
        out[3] = a.upperBound.y;
    }
}
void rw_joint_reaction(void* h, int ji, float inv_dt, float* out)
{
    const b2Joint* j = static_cast<RefWorld*>(h)->joints[ji];
    const b2Vec2 F = j->GetReactionForce(inv_dt);
    out[0] = F.x;
    out[1] = F.y;
    out[2] = j->GetReactionTorque(inv_dt);
}
// joint setters through the reference's own classes; 1 when the joint type has no such setter
int rw_joint_set(void* h, int ji, int prop, const float* v)
{
    b2Joint* j = static_cast<RefWorld*>(h)->joints[ji];
    const b2JointType t = j->GetType();
    const bool flag = v[0] != 0.0f;
    if (t == e_revoluteJoint) {
        b2RevoluteJoint* r = static_cast<b2RevoluteJoint*>(j);
        switch (prop) {
        case 0: r->SetMotorSpeed(v[0]); return 0;
        case 1: r->SetMaxMotorTorque(v[0]); return 0;
        case 2: r->EnableMotor(flag); return 0;
        case 3: r->EnableLimit(flag); return 0;
        case 4: r->SetLimits(v[0], v[1]); return 0;
        default: return 1;
        }
    }
    if (t == e_prismaticJoint) {
        b2PrismaticJoint* p = static_cast<b2PrismaticJoint*>(j);
        switch (prop) {
        case 0: p->SetMotorSpeed(v[0]); return 0;
        case 1: p->SetMaxMotorForce(v[0]); return 0;
        case 2: p->EnableMotor(flag); return 0;
        case 3: p->EnableLimit(flag); return 0;
        case 4: p->SetLimits(v[0], v[1]); return 0;
        default: return 1;
        }
    }
    if (t == e_wheelJoint) {
        b2WheelJoint* w = static_cast<b2WheelJoint*>(j);
        switch (prop) {
        case 0: w->SetMotorSpeed(v[0]); return 0;
        case 1: w->SetMaxMotorTorque(v[0]); return 0;
        case 2: w->EnableMotor(flag); return 0;
        case 6: w->SetSpringFrequencyHz(v[0]); return 0;
        case 7: w->SetSpringDampingRatio(v[0]); return 0;
        default: return 1;
        }
    }
    if (t == e_distanceJoint) {
        b2DistanceJoint* d = static_cast<b2DistanceJoint*>(j);
        switch (prop) {
        case 5: d->SetLength(v[0]); return 0;
        case 6: d->SetFrequency(v[0]); return 0;
        case 7: d->SetDampingRatio(v[0]); return 0;
        default: return 1;
        }
    }
    if (t == e_weldJoint) {
        b2WeldJoint* d = static_cast<b2WeldJoint*>(j);
        if (prop == 6) { d->SetFrequency(v[0]); return 0; }
        if (prop == 7) { d->SetDampingRatio(v[0]); return 0; }
        return 1;
    }
    if (t == e_mouseJoint) {
        b2MouseJoint* m = static_cast<b2MouseJoint*>(j);
        if (prop == 6) { m->SetFrequency(v[0]); return 0; }
        if (prop == 7) { m->SetDampingRatio(v[0]); return 0; }
        if (prop == 9) { m->SetMaxForce(v[0]); return 0; }
        return 1;
    }
    if (t == e_ropeJoint && prop == 8) { static_cast<b2RopeJoint*>(j)->SetMaxLength(v[0]); return 0; }
    if (t == e_frictionJoint) {
        b2FrictionJoint* f = static_cast<b2FrictionJoint*>(j);
        if (prop == 9) { f->SetMaxForce(v[0]); return 0; }
        if (prop == 10) { f->SetMaxTorque(v[0]); return 0; }
        return 1;
    }
    if (t == e_motorJoint) {
        b2MotorJoint* m = static_cast<b2MotorJoint*>(j);
        switch (prop) {
        case 9: m->SetMaxForce(v[0]); return 0;
        case 10: m->SetMaxTorque(v[0]); return 0;
        case 11: m->SetLinearOffset(b2Vec2(v[0], v[1])); return 0;
        case 12: m->SetAngularOffset(v[0]); return 0;
        case 13: m->SetCorrectionFactor(v[0]); return 0;
        default: return 1;
        }
    }
    if (t == e_gearJoint && prop == 14) { static_cast<b2GearJoint*>(j)->SetRatio(v[0]); return 0; }
    return 1;
}
void rw_shift_origin(void* h, float x, float y)
{
    static_cast<RefWorld*>(h)->world.ShiftOrigin(b2Vec2(x, y));
}
void rw_fixture_set(void* h, int f, int prop, const float* v)
{
    b2Fixture* fx = static_cast<RefWorld*>(h)->fixtures[f];
    switch (prop) {
    case 0: fx->SetFriction(v[0]); break;
    case 1: fx->SetRestitution(v[0]); break;
    case 2: fx->SetDensity(v[0]); break;
    case 3: fx->SetSensor(v[0] != 0.0f); break;
    case 4: {
        b2Filter filter;
        filter.categoryBits = (uint16)(int)v[0];
        filter.maskBits = (uint16)(int)v[1];
        filter.groupIndex = (int16)(int)v[2];
        fx->SetFilterData(filter);
        break;
    }
    default: break;
    }
}
void rw_body_info(void* h, int bi, float* out, int* flags)
{
    const b2Body* b = static_cast<RefWorld*>(h)->bodies[bi];
    out[0] = b->GetMass();
    out[1] = b->GetInertia();
    out[2] = b->GetLocalCenter().x;
    out[3] = b->GetLocalCenter().y;
    out[4] = b->GetLinearDamping();
    out[5] = b->GetAngularDamping();
    out[6] = b->GetGravityScale();
    *flags = (int)b->GetType() | (b->IsBullet() ? 4 : 0) | (b->IsFixedRotation() ? 8 : 0) |
             (b->IsSleepingAllowed() ? 16 : 0) | (b->IsActive() ? 32 : 0);
}
void rw_tree_stats(void* h, int* height, int* balance, float* quality)
{
    const b2World& w = static_cast<RefWorld*>(h)->world;
    *height = w.GetTreeHeight();
    *balance = w.GetTreeBalance();
    *quality = w.GetTreeQuality();
}
void rw_clear_forces(void* h)
{
    static_cast<RefWorld*>(h)->world.ClearForces();
}
void rw_set_presolve_rule(void* h, const int* bits, int n)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->rule.bits.assign(bits, bits + n);
    w->world.SetContactListener(&w->rule);
}
int rw_destroy_body(void* h, int b, int* calls, int cap)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    b2Body* body = w->bodies[b];
    w->goodbye.calls.clear();
    w->world.DestroyBody(body);
    ForgetDestroyed(w, body);
    return TakeGoodbyes(w, calls, cap);
}
int rw_destroy_joint(void* h, int j, int* calls, int cap)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->goodbye.calls.clear();
    w->world.DestroyJoint(w->joints[j]);
    ForgetDestroyed(w, nullptr);
    return TakeGoodbyes(w, calls, cap);
}
int rw_destroy_fixture(void* h, int f, int* calls, int cap)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    w->goodbye.calls.clear();
    b2Fixture* fx = w->fixtures[f];
    fx->GetBody()->DestroyFixture(fx);
    ForgetDestroyed(w, nullptr);
    return TakeGoodbyes(w, calls, cap);
}
int rw_contact_count(void* h) { return static_cast<RefWorld*>(h)->world.GetContactCount(); }

// Per body (creation order), 12 floats: xf.p.x, xf.p.y, sweep.a, sweep.c.x, sweep.c.y, v.x, v.y, w,
// xf.q.s, xf.q.c, sleepTime, awake (0/1)
void rw_get_bodies(void* h, float* out)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    for (size_t i = 0; i < w->bodies.size(); ++i) {
        const b2Body* b = w->bodies[i];
        float* o = out + 12 * i;
        if (!b) {
            std::memset(o, 0, 12 * sizeof(float));
            continue;
        }
        o[0] = b->m_xf.p.x; o[1] = b->m_xf.p.y; o[2] = b->m_sweep.a;
        o[3] = b->m_sweep.c.x; o[4] = b->m_sweep.c.y;
        o[5] = b->m_linearVelocity.x; o[6] = b->m_linearVelocity.y; o[7] = b->m_angularVelocity;
        o[8] = b->m_xf.q.s; o[9] = b->m_xf.q.c; o[10] = b->m_sleepTime;
        o[11] = b->IsAwake() ? 1.0f : 0.0f;
    }
}

// A chain fixture from consecutive edge records flagged as chain children (s[10]: 1 the first
// child, 2 each next one): b2ChainShape::CreateChain over the children's first vertices and the last
// child's second, the first child's ghost vertex as prevVertex and the last child's as nextVertex
// (for a closed chain this equals b2ChainShape::CreateLoop). One b2Fixture stands for the records;
// their ids are its first id + the child index.
int rw_chain(void* h, int body, int nchild, const float* s, const float* mat, const int* filt)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    std::vector<b2Vec2> v((size_t)nchild + 1);
    for (int i = 0; i < nchild; ++i) v[i].Set(s[16 * i], s[16 * i + 1]);
    const float* first = s;
    const float* last = s + 16 * (nchild - 1);
    v[nchild].Set(last[2], last[3]);
    b2ChainShape chain;
    chain.CreateChain(v.data(), nchild + 1);
    if (first[8] != 0.0f) chain.SetPrevVertex(b2Vec2(first[4], first[5]));
    if (last[9] != 0.0f) chain.SetNextVertex(b2Vec2(last[6], last[7]));
    b2FixtureDef fd;
    fd.shape = &chain;
    fd.density = mat[0];
    fd.friction = mat[1];
    fd.restitution = mat[2];
    fd.filter.categoryBits = (uint16)filt[0];
    fd.filter.maskBits = (uint16)filt[1];
    fd.filter.groupIndex = (int16)filt[2];
    fd.isSensor = filt[3] != 0;
    const int id = (int)w->fixtures.size();
    fd.userData = (void*)(intptr_t)(id + 1);
    b2Fixture* fx = w->bodies[body]->CreateFixture(&fd);
    for (int i = 0; i < nchild; ++i) w->fixtures.push_back(fx);
    return id;
}

// Contacts in world-list order. ints (8 per contact): fixtureA, fixtureB, flags, pointCount,
// manifold type, id0 key, id1 key, toiCount. floats (12 per contact): localNormal.xy,
// localPoint.xy, then per point: localPoint.xy, normalImpulse, tangentImpulse.
int rw_get_contacts(void* h, int* ints, float* flts, int cap)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    int n = 0;
    for (b2Contact* c = w->world.GetContactList(); c; c = c->GetNext()) {
        if (n < cap) {
            int* i = ints + 8 * n;
            float* f = flts + 12 * n;
            const b2Manifold& m = c->m_manifold;
            i[0] = fixture_index(c->m_fixtureA) + c->GetChildIndexA();
            i[1] = fixture_index(c->m_fixtureB) + c->GetChildIndexB();
            i[2] = (int)c->m_flags; i[3] = m.pointCount; i[4] = m.pointCount > 0 ? (int)m.type : 0;
            i[5] = m.pointCount > 0 ? (int)m.points[0].id.key : 0;
            i[6] = m.pointCount > 1 ? (int)m.points[1].id.key : 0;
            i[7] = c->m_toiCount;
            // manifold fields are dead when pointCount == 0 (a collide may return early leaving them stale)
            bool any = m.pointCount > 0;
            f[0] = any ? m.localNormal.x : 0.0f; f[1] = any ? m.localNormal.y : 0.0f;
            f[2] = any ? m.localPoint.x : 0.0f; f[3] = any ? m.localPoint.y : 0.0f;
            for (int p = 0; p < 2; ++p) {
                bool on = p < m.pointCount;
                f[4 + 4 * p] = on ? m.points[p].localPoint.x : 0.0f;
                f[5 + 4 * p] = on ? m.points[p].localPoint.y : 0.0f;
                f[6 + 4 * p] = on ? m.points[p].normalImpulse : 0.0f;
                f[7 + 4 * p] = on ? m.points[p].tangentImpulse : 0.0f;
            }
        }
        ++n;
    }
    return n;
}

// Per fixture (creation order): proxy id and the broadphase fat AABB (lower.xy, upper.xy).
void rw_get_proxies(void* h, int* proxyIds, float* fat)
{
    RefWorld* w = static_cast<RefWorld*>(h);
    const b2BroadPhase& bp = w->world.m_contactManager.m_broadPhase;
    for (size_t i = 0; i < w->fixtures.size(); ++i) {
        const b2Fixture* f = w->fixtures[i];
        int id = f && f->m_proxyCount > 0 ? f->m_proxies[0].proxyId : -1;
        proxyIds[i] = id;
        if (id >= 0) {
            const b2AABB& a = bp.GetFatAABB(id);
            fat[4 * i] = a.lowerBound.x; fat[4 * i + 1] = a.lowerBound.y;
            fat[4 * i + 2] = a.upperBound.x; fat[4 * i + 3] = a.upperBound.y;
        }
    }
}

// Direct narrowphase call (b2Collide* from Collision/b2CollidePolygon.cpp, b2CollideCircle.cpp,
// b2CollideEdge.cpp). Shapes use the rw_fixture encoding; xf = {p.x, p.y, q.s, q.c}.
// Output: ints {type, pointCount, id0, id1}; floats as rw_get_contacts (impulses zero).
int rw_collide(int typeA, const float* sA, int nA, const float* xfA,
               int typeB, const float* sB, int nB, const float* xfB, int* oi, float* of)
{
    b2CircleShape cA, cB; b2EdgeShape eA; b2PolygonShape pA, pB;
    auto make_poly = [](b2PolygonShape& p, int type, const float* s, int n) {
        if (type == 3) { if (n == 5) p.SetAsBox(s[0], s[1], b2Vec2(s[2], s[3]), s[4]); else p.SetAsBox(s[0], s[1]); }
        else { b2Vec2 pts[8]; for (int i = 0; i < n && i < 8; ++i) pts[i].Set(s[2*i], s[2*i+1]); p.Set(pts, n); }
    };
    b2Transform xa, xb;
    xa.p.Set(xfA[0], xfA[1]); xa.q.s = xfA[2]; xa.q.c = xfA[3];
    xb.p.Set(xfB[0], xfB[1]); xb.q.s = xfB[2]; xb.q.c = xfB[3];
    b2Manifold m;
    m.pointCount = 0;
    bool polyA = typeA == 2 || typeA == 3, polyB = typeB == 2 || typeB == 3;
    if (typeA == 0 && typeB == 0) {
        cA.m_p.Set(sA[0], sA[1]); cA.m_radius = sA[2]; cB.m_p.Set(sB[0], sB[1]); cB.m_radius = sB[2];
        b2CollideCircles(&m, &cA, xa, &cB, xb);
    } else if (polyA && typeB == 0) {
        make_poly(pA, typeA, sA, nA); cB.m_p.Set(sB[0], sB[1]); cB.m_radius = sB[2];
        b2CollidePolygonAndCircle(&m, &pA, xa, &cB, xb);
    } else if (polyA && polyB) {
        make_poly(pA, typeA, sA, nA); make_poly(pB, typeB, sB, nB);
        b2CollidePolygons(&m, &pA, xa, &pB, xb);
    } else if (typeA == 1 && (typeB == 0 || polyB)) {
        eA.Set(b2Vec2(sA[0], sA[1]), b2Vec2(sA[2], sA[3]));
        eA.m_vertex0.Set(sA[4], sA[5]); eA.m_vertex3.Set(sA[6], sA[7]);
        eA.m_hasVertex0 = sA[8] != 0.0f; eA.m_hasVertex3 = sA[9] != 0.0f;
        if (typeB == 0) { cB.m_p.Set(sB[0], sB[1]); cB.m_radius = sB[2]; b2CollideEdgeAndCircle(&m, &eA, xa, &cB, xb); }
        else { make_poly(pB, typeB, sB, nB); b2CollideEdgeAndPolygon(&m, &eA, xa, &pB, xb); }
    } else {
        return -1;
    }
    oi[0] = m.pointCount > 0 ? (int)m.type : 0; // type is left unset when the shapes do not touch
    oi[1] = m.pointCount;
    oi[2] = m.pointCount > 0 ? (int)m.points[0].id.key : 0;
    oi[3] = m.pointCount > 1 ? (int)m.points[1].id.key : 0;
    of[0] = m.pointCount > 0 ? m.localNormal.x : 0.0f; of[1] = m.pointCount > 0 ? m.localNormal.y : 0.0f;
    of[2] = m.pointCount > 0 ? m.localPoint.x : 0.0f; of[3] = m.pointCount > 0 ? m.localPoint.y : 0.0f;
    for (int p = 0; p < 2; ++p) {
        bool on = p < m.pointCount;
        of[4 + 4 * p] = on ? m.points[p].localPoint.x : 0.0f;
        of[5 + 4 * p] = on ? m.points[p].localPoint.y : 0.0f;
        of[6 + 4 * p] = 0.0f; of[7 + 4 * p] = 0.0f;
    }
    return 0;
}

// Polygon construction as the reference does it (b2PolygonShape::Set / SetAsBox and ComputeMass):
// out = {count, vertices (16), normals (16), centroid (2), mass, center (2), I} for density 1.
void rw_polygon(int type, const float* s, int n, float density, float* out)
{
    b2PolygonShape p;
    if (type == 3) { if (n == 5) p.SetAsBox(s[0], s[1], b2Vec2(s[2], s[3]), s[4]); else p.SetAsBox(s[0], s[1]); }
    else { b2Vec2 pts[8]; for (int i = 0; i < n && i < 8; ++i) pts[i].Set(s[2*i], s[2*i+1]); p.Set(pts, n); }
    std::memset(out, 0, sizeof(float) * 40);
    out[0] = (float)p.m_count;
    for (int i = 0; i < p.m_count; ++i) {
        out[1 + 2 * i] = p.m_vertices[i].x; out[2 + 2 * i] = p.m_vertices[i].y;
        out[17 + 2 * i] = p.m_normals[i].x; out[18 + 2 * i] = p.m_normals[i].y;
    }
    out[33] = p.m_centroid.x; out[34] = p.m_centroid.y;
    b2MassData md;
    p.ComputeMass(&md, density);
    out[35] = md.mass; out[36] = md.center.x; out[37] = md.center.y; out[38] = md.I;
}

// b2TimeOfImpact (Collision/b2TimeOfImpact.cpp:257) on two shapes and sweeps.
// sweep = {localCenter.xy, c0.xy, c.xy, a0, a, alpha0}; out = {state, t}.
void rw_toi(int typeA, const float* sA, int nA, const float* swA,
            int typeB, const float* sB, int nB, const float* swB, float tMax, float* out)
{
    b2CircleShape cA, cB; b2EdgeShape eA; b2PolygonShape pA, pB;
    auto make = [&](int type, const float* s, int n, b2CircleShape& c, b2PolygonShape& p, b2EdgeShape* e) -> const b2Shape* {
        if (type == 0) { c.m_p.Set(s[0], s[1]); c.m_radius = s[2]; return &c; }
        if (type == 1 && e) { e->Set(b2Vec2(s[0], s[1]), b2Vec2(s[2], s[3])); return e; }
        if (type == 3) { if (n == 5) p.SetAsBox(s[0], s[1], b2Vec2(s[2], s[3]), s[4]); else p.SetAsBox(s[0], s[1]); return &p; }
        b2Vec2 pts[8]; for (int i = 0; i < n && i < 8; ++i) pts[i].Set(s[2*i], s[2*i+1]); p.Set(pts, n); return &p;
    };
    b2TOIInput in;
    in.proxyA.Set(make(typeA, sA, nA, cA, pA, &eA), 0);
    in.proxyB.Set(make(typeB, sB, nB, cB, pB, nullptr), 0);
    auto sw = [](b2Sweep& s, const float* f) {
        s.localCenter.Set(f[0], f[1]); s.c0.Set(f[2], f[3]); s.c.Set(f[4], f[5]);
        s.a0 = f[6]; s.a = f[7]; s.alpha0 = f[8];
    };
    sw(in.sweepA, swA); sw(in.sweepB, swB);
    in.tMax = tMax;
    b2TOIOutput o;
    b2TimeOfImpact(&o, &in);
    out[0] = (float)o.state; out[1] = o.t;
}

void rw_sincosf(float x, float* s, float* c) { b2Rot q(x); *s = q.s; *c = q.c; }

// b2World::QueryAABB: the fixtures the reference reports for the box, sorted by creation index.
int rw_query_aabb(void* h, const float* box, int* out, int cap)
{
    struct Collect : b2QueryCallback {
        std::vector<int> hits;
        bool ReportFixture(b2Fixture* f) override { hits.push_back(fixture_index(f)); return true; }
    } cb;
    b2AABB aabb;
    aabb.lowerBound.Set(box[0], box[1]);
    aabb.upperBound.Set(box[2], box[3]);
    static_cast<RefWorld*>(h)->world.QueryAABB(&cb, aabb);
    std::sort(cb.hits.begin(), cb.hits.end());
    for (int i = 0; i < (int)cb.hits.size() && i < cap; ++i) out[i] = cb.hits[i];
    return (int)cb.hits.size();
}

// b2World::RayCast with a closest-hit callback (returns each reported fraction): the last report.
int rw_raycast(void* h, const float* ray, float* hit)
{
    struct Closest : b2RayCastCallback {
        int fixture = -1;
        float out[5] = {0, 0, 0, 0, 0};
        float32 ReportFixture(b2Fixture* f, const b2Vec2& point, const b2Vec2& normal, float32 fraction) override
        {
            fixture = fixture_index(f);
            out[0] = fraction; out[1] = point.x; out[2] = point.y; out[3] = normal.x; out[4] = normal.y;
            return fraction;
        }
    } cb;
    static_cast<RefWorld*>(h)->world.RayCast(&cb, b2Vec2(ray[0], ray[1]), b2Vec2(ray[2], ray[3]));
    for (int i = 0; i < 5; ++i) hit[i] = cb.out[i];
    return cb.fixture;
}

// Steps many independent reference worlds on `threads` host threads. The reference fills its
// contact-type registry lazily on the first b2Contact::Create (Dynamics/Contacts/b2Contact.cpp:74-78),
// so one contact is created on the calling thread first.
void rw_step_many(void** hs, int n, float dt, int vi, int pi, int steps, int threads)
{
    {
        b2World warm(b2Vec2(0.0f, -10.0f));
        b2BodyDef bd;
        bd.type = b2_dynamicBody;
        b2CircleShape c;
        c.m_radius = 1.0f;
        warm.CreateBody(&bd)->CreateFixture(&c, 1.0f);
        warm.CreateBody(&bd)->CreateFixture(&c, 1.0f);
        warm.Step(1.0f / 60.0f, 1, 1);
    }
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([=]() {
            for (int i = t; i < n; i += threads)
                for (int s = 0; s < steps; ++s) static_cast<RefWorld*>(hs[i])->world.Step(dt, vi, pi);
        });
    }
    for (std::thread& th : pool) th.join();
}

} // extern "C"
