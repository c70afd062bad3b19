// Oracle (test infrastructure only): C-ABI of the CPU restatement, mirroring oracle/ref_driver.cpp
// function by function (po_* here, rw_* there) so the same Python scene builder drives both.
#include "world.h"

#include <cstring>
#include <thread>
#include <vector>

using namespace b2o;

namespace {
Shape MakeShape(int type, const float* s, int n)
{
    Shape sh;
    switch (type) {
    case 0:
        sh.type = kCircle; sh.p = V(s[0], s[1]); sh.radius = s[2];
        break;
    case 1:
        sh.type = kEdge; sh.radius = kPolygonRadius;
        sh.v1 = V(s[0], s[1]); sh.v2 = V(s[2], s[3]); sh.v0 = V(s[4], s[5]); sh.v3 = V(s[6], s[7]);
        sh.hasV0 = s[8] != 0.0f; sh.hasV3 = s[9] != 0.0f;
        sh.chain = (int)s[10];
        break;
    case 2: {
        Vec2 pts[kMaxPolygonVertices];
        int m = n < kMaxPolygonVertices ? n : kMaxPolygonVertices;
        for (int i = 0; i < m; ++i) pts[i] = V(s[2 * i], s[2 * i + 1]);
        PolygonSet(sh, pts, n);
        break;
    }
    default:
        if (n == 5) PolygonSetAsBox(sh, s[0], s[1], V(s[2], s[3]), s[4]);
        else PolygonSetAsBox(sh, s[0], s[1]);
        break;
    }
    return sh;
}
} // namespace

extern "C" {

void po_set_trig(int mode) { g_trig_mode = mode; }
void* po_create(float gx, float gy) { World* w = new World(); w->gravity = V(gx, gy); return w; }
void po_destroy(void* h) { delete static_cast<World*>(h); }
void po_config(void* h, int allowSleep, int warmStarting, int continuous, int subStepping)
{
    World* w = static_cast<World*>(h);
    if ((allowSleep != 0) != w->allowSleep) {
        w->allowSleep = allowSleep != 0;
        if (!w->allowSleep)
            for (int b = w->bodyList; b != kNull; b = w->bodies[b].next) w->SetAwake(b, true);
    }
    w->warmStarting = warmStarting != 0;
    w->continuous = continuous != 0;
    w->subStepping = subStepping != 0;
}
void po_record_events(void* h, int on) { static_cast<World*>(h)->recordEvents = on != 0; }
int po_body(void* h, int type, const float* f, int flags) { return static_cast<World*>(h)->CreateBody(type, f, flags); }
int po_fixture(void* h, int body, int shapeType, const float* s, int n, const float* mat, const int* filt)
{
    World* w = static_cast<World*>(h);
    return w->CreateFixture(body, MakeShape(shapeType, s, n), mat[0], mat[1], mat[2], filt[0], filt[1], filt[2], filt[3] != 0);
}
int po_revolute(void* h, int a, int b, const float* f, int flags) { return static_cast<World*>(h)->CreateRevolute(a, b, f, flags); }
int po_joint(void* h, int type, int a, int b, const float* f, int flags) { return static_cast<World*>(h)->CreateJoint(type, a, b, f, flags); }
// Bulk scene build: body b is created, then its fixtures (fbody is non-decreasing), then all joints.
void po_build(void* h, int nb, const int* btype, const float* bf, const int* bflags, int nf, const int* fbody,
              const int* ftype, const float* fshape, const int* fn, const float* fmat, const int* ffilt, int nj,
              const int* ja, const int* jb, const float* jf, const int* jflags)
{
    int fi = 0;
    for (int b = 0; b < nb; ++b) {
        po_body(h, btype[b], bf + 9 * b, bflags[b]);
        while (fi < nf && fbody[fi] == b) {
            po_fixture(h, b, ftype[fi], fshape + 16 * fi, fn[fi], fmat + 3 * fi, ffilt + 4 * fi);
            ++fi;
        }
    }
    for (int j = 0; j < nj; ++j) po_revolute(h, ja[j], jb[j], jf + 12 * j, jflags[j]);
}

void po_step(void* h, float dt, int vi, int pi) { static_cast<World*>(h)->Step(dt, vi, pi); }
void po_body_edit(void* h, int op, int body, int wake, const float* v) { static_cast<World*>(h)->ApplyEdit(op, body, wake, v); }

// Steps many independent worlds on `threads` host threads (static round-robin split of the worlds,
// which the caller orders by estimated cost). Used for the all-cores CPU baseline.
void po_step_many(void** hs, int n, float dt, int vi, int pi, int steps, int threads);
int po_body_count(void* h) { return (int)static_cast<World*>(h)->bodies.size(); }
// b2World::DestroyBody / DestroyJoint, b2Body::DestroyFixture; the destruction listener's calls
// {0 joint / 1 fixture, index} of the call go to calls (2 ints each, up to cap), their count returned
static int Goodbyes(World* w, int* calls, int cap)
{
    const int n = (int)w->goodbyes.size();
    for (int i = 0; i < n && i < cap; ++i) { calls[2 * i] = w->goodbyes[i].first; calls[2 * i + 1] = w->goodbyes[i].second; }
    return n;
}
void po_set_filter_rule(void* h, int modulus, int firstOther)
{
    World* w = static_cast<World*>(h);
    w->filterModulus = modulus;
    w->filterStatic = firstOther;
}
// b2World::SetGravity, SetAllowSleeping (b2World.cpp:370-385: turning sleep off wakes every body of
// the list), SetWarmStarting, SetContinuousPhysics, SetSubStepping, SetAutoClearForces
void po_set_settings(void* h, float gx, float gy, int allowSleep, int warm, int continuous, int subStepping,
                     int autoClear)
{
    World* w = static_cast<World*>(h);
    w->gravity = V(gx, gy);
    if (w->allowSleep && !allowSleep)
        for (int b = w->bodyList; b != kNull; b = w->bodies[b].next) w->SetAwake(b, true);
    w->allowSleep = allowSleep != 0;
    w->warmStarting = warm != 0;
    w->continuous = continuous != 0;
    w->subStepping = subStepping != 0;
    if (autoClear) w->wflags |= 0x4u;
    else w->wflags &= ~0x4u;
}
// b2Joint::GetReactionForce and GetReactionTorque of every joint type (Dynamics/Joints/*.cpp), with
// the reference's operation order: out = force x, force y, torque
void po_joint_reaction(void* h, int ji, float inv_dt, float* out)
{
    const Joint& j = static_cast<World*>(h)->joints[ji];
    Vec2 F = V(0.0f, 0.0f);
    float T = 0.0f;
    switch (j.type) {
    case kRevoluteJoint:
    case kWeldJoint:
    case kFrictionJoint:
    case kMotorJoint:
        F = V(inv_dt * j.impulse[0], inv_dt * j.impulse[1]);
        T = inv_dt * j.impulse[2];
        break;
    case kPrismaticJoint: {
        const float k = j.motorImpulse + j.impulse[2];
        F = V(inv_dt * (j.impulse[0] * j.perp.x + k * j.u.x), inv_dt * (j.impulse[0] * j.perp.y + k * j.u.y));
        T = inv_dt * j.impulse[1];
        break;
    }
    case kDistanceJoint:
    case kRopeJoint: {
        const float s = inv_dt * j.impulse[0];
        F = V(s * j.u.x, s * j.u.y);
        break;
    }
    case kWheelJoint:
        F = V(inv_dt * (j.impulse[0] * j.ay.x + j.springImpulse * j.ax.x),
              inv_dt * (j.impulse[0] * j.ay.y + j.springImpulse * j.ax.y));
        T = inv_dt * j.motorImpulse;
        break;
    case kMouseJoint:
        F = V(inv_dt * j.impulse[0], inv_dt * j.impulse[1]);
        T = inv_dt * 0.0f;
        break;
    case kPulleyJoint:
        F = V(inv_dt * (j.impulse[0] * j.uB.x), inv_dt * (j.impulse[0] * j.uB.y));
        break;
    case kGearJoint:
        F = V(inv_dt * (j.impulse[0] * j.JvAC.x), inv_dt * (j.impulse[0] * j.JvAC.y));
        T = inv_dt * (j.impulse[0] * j.JwA);
        break;
    default: break;
    }
    out[0] = F.x;
    out[1] = F.y;
    out[2] = T;
}
int po_joint_set(void* h, int j, int prop, const float* v)
{
    return static_cast<World*>(h)->SetJointProperty(j, prop, v);
}
void po_shift_origin(void* h, float x, float y)
{
    static_cast<World*>(h)->ShiftOrigin(V(x, y));
}
void po_fixture_set(void* h, int f, int prop, const float* v)
{
    static_cast<World*>(h)->SetFixtureProperty(f, prop, v);
}
void po_body_set(void* h, int b, int prop, const float* v)
{
    static_cast<World*>(h)->SetBodyProperty(b, prop, v);
}
// b2Body::GetMass, GetInertia, GetLocalCenter, damping, gravity scale and flags (b2Body.h:227-682)
void po_body_info(void* h, int bi, float* out, int* flags)
{
    const Body& b = static_cast<World*>(h)->bodies[bi];
    out[0] = b.mass;
    out[1] = b.I + b.mass * Dot(b.sweep.localCenter, b.sweep.localCenter);
    out[2] = b.sweep.localCenter.x;
    out[3] = b.sweep.localCenter.y;
    out[4] = b.linearDamping;
    out[5] = b.angularDamping;
    out[6] = b.gravityScale;
    *flags = b.type | ((b.flags & kBBullet) ? 4 : 0) | ((b.flags & kBFixedRot) ? 8 : 0) |
             ((b.flags & kBAutoSleep) ? 16 : 0) | ((b.flags & kBActive) ? 32 : 0);
}
// b2World::GetTreeHeight, GetTreeBalance, GetTreeQuality (b2World.cpp:1246-1259)
void po_tree_stats(void* h, int* height, int* balance, float* quality)
{
    const Tree& t = static_cast<World*>(h)->bp.tree;
    *height = t.Height();
    *balance = t.MaxBalance();
    *quality = t.AreaRatio();
}
// b2World::ClearForces (b2World.cpp:967-974)
void po_clear_forces(void* h)
{
    World* w = static_cast<World*>(h);
    for (int b = w->bodyList; b != kNull; b = w->bodies[b].next) {
        w->bodies[b].force = V(0.0f, 0.0f);
        w->bodies[b].torque = 0.0f;
    }
}
void po_set_presolve_rule(void* h, const int* bits, int n)
{
    World* w = static_cast<World*>(h);
    w->preSolveRule.assign(bits, bits + n);
}
int po_destroy_body(void* h, int b, int* calls, int cap)
{
    World* w = static_cast<World*>(h);
    w->DestroyBody(b);
    return Goodbyes(w, calls, cap);
}
int po_destroy_joint(void* h, int j, int* calls, int cap)
{
    World* w = static_cast<World*>(h);
    w->goodbyes.clear();
    w->DestroyJoint(j);
    return Goodbyes(w, calls, cap);
}
int po_destroy_fixture(void* h, int f, int* calls, int cap)
{
    World* w = static_cast<World*>(h);
    w->DestroyFixture(f);
    return Goodbyes(w, calls, cap);
}
int po_contact_count(void* h) { return static_cast<World*>(h)->contactCount; }

void po_get_bodies(void* h, float* out)
{
    World* w = static_cast<World*>(h);
    for (size_t i = 0; i < w->bodies.size(); ++i) {
        const Body& b = w->bodies[i];
        float* o = out + 12 * i;
        if (!b.alive) {
            std::memset(o, 0, 12 * sizeof(float));
            continue;
        }
        o[0] = b.xf.p.x; o[1] = b.xf.p.y; o[2] = b.sweep.a;
        o[3] = b.sweep.c.x; o[4] = b.sweep.c.y;
        o[5] = b.v.x; o[6] = b.v.y; o[7] = b.w;
        o[8] = b.xf.q.s; o[9] = b.xf.q.c; o[10] = b.sleepTime;
        o[11] = b.IsAwake() ? 1.0f : 0.0f;
    }
}

int po_get_contacts(void* h, int* ints, float* flts, int cap)
{
    World* w = static_cast<World*>(h);
    int n = 0;
    for (int c = w->contactList; c != kNull; c = w->contacts[c].next) {
        if (n < cap) {
            const Contact& ct = w->contacts[c];
            const Manifold& m = ct.m;
            int* i = ints + 8 * n;
            float* f = flts + 12 * n;
            i[0] = ct.fA; i[1] = ct.fB; i[2] = (int)ct.flags; i[3] = m.pointCount; i[4] = m.pointCount > 0 ? m.type : 0;
            i[5] = m.pointCount > 0 ? (int)m.points[0].id : 0;
            i[6] = m.pointCount > 1 ? (int)m.points[1].id : 0;
            i[7] = ct.toiCount;
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

void po_get_proxies(void* h, int* proxyIds, float* fat)
{
    World* w = static_cast<World*>(h);
    for (size_t i = 0; i < w->fixtures.size(); ++i) {
        const Fixture& f = w->fixtures[i];
        proxyIds[i] = f.proxyCount > 0 ? f.proxyId : -1;
        if (f.proxyCount > 0) {
            const AABB& a = w->bp.FatAABB(f.proxyId);
            fat[4 * i] = a.lo.x; fat[4 * i + 1] = a.lo.y; fat[4 * i + 2] = a.hi.x; fat[4 * i + 3] = a.hi.y;
        }
    }
}

// Every UpdatePairs list of the last step as (proxyA, proxyB) with (-1, -1) after each list.
int po_get_pairs(void* h, int* out, int cap)
{
    World* w = static_cast<World*>(h);
    int n = (int)w->stepPairs.size();
    for (int i = 0; i < n && i < cap; ++i) { out[2 * i] = w->stepPairs[i].a; out[2 * i + 1] = w->stepPairs[i].b; }
    return n;
}

// Listener events of the last step: ints {kind, fixtureA, fixtureB}, floats {n0, n1, t0, t1}.
int po_get_events(void* h, int* ints, float* flts, int cap)
{
    World* w = static_cast<World*>(h);
    int n = (int)w->events.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const Event& e = w->events[i];
        ints[3 * i] = e.kind; ints[3 * i + 1] = e.fA; ints[3 * i + 2] = e.fB;
        flts[4 * i] = e.n0; flts[4 * i + 1] = e.n1; flts[4 * i + 2] = e.t0; flts[4 * i + 3] = e.t1;
    }
    return n;
}

int po_collide(int typeA, const float* sA, int nA, const float* xfA, int typeB, const float* sB, int nB,
               const float* xfB, int* oi, float* of)
{
    Shape a = MakeShape(typeA, sA, nA), b = MakeShape(typeB, sB, nB);
    Xf xa, xb;
    xa.p = V(xfA[0], xfA[1]); xa.q.s = xfA[2]; xa.q.c = xfA[3];
    xb.p = V(xfB[0], xfB[1]); xb.q.s = xfB[2]; xb.q.c = xfB[3];
    Manifold m;
    m.pointCount = 0;
    bool polyA = a.type == kPolygon, polyB = b.type == kPolygon;
    if (a.type == kCircle && b.type == kCircle) CollideCircles(&m, a, xa, b, xb);
    else if (polyA && b.type == kCircle) CollidePolygonAndCircle(&m, a, xa, b, xb);
    else if (polyA && polyB) CollidePolygons(&m, a, xa, b, xb);
    else if (a.type == kEdge && b.type == kCircle) CollideEdgeAndCircle(&m, a, xa, b, xb);
    else if (a.type == kEdge && polyB) CollideEdgeAndPolygon(&m, a, xa, b, xb);
    else return -1;
    oi[0] = m.pointCount > 0 ? m.type : 0; // type is left unset when the shapes do not touch
    oi[1] = m.pointCount;
    oi[2] = m.pointCount > 0 ? (int)m.points[0].id : 0;
    oi[3] = m.pointCount > 1 ? (int)m.points[1].id : 0;
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

void po_polygon(int type, const float* s, int n, float density, float* out)
{
    Shape p = MakeShape(type, s, n);
    std::memset(out, 0, sizeof(float) * 40);
    out[0] = (float)p.count;
    for (int i = 0; i < p.count; ++i) {
        out[1 + 2 * i] = p.verts[i].x; out[2 + 2 * i] = p.verts[i].y;
        out[17 + 2 * i] = p.normals[i].x; out[18 + 2 * i] = p.normals[i].y;
    }
    out[33] = p.centroid.x; out[34] = p.centroid.y;
    MassData md;
    ComputeMass(p, density, &md);
    out[35] = md.mass; out[36] = md.center.x; out[37] = md.center.y; out[38] = md.I;
}

void po_toi(int typeA, const float* sA, int nA, const float* swA, int typeB, const float* sB, int nB,
            const float* swB, float tMax, float* out)
{
    Shape a = MakeShape(typeA, sA, nA), b = MakeShape(typeB, sB, nB);
    DistanceProxy pa, pb;
    ProxyOf(&pa, a);
    ProxyOf(&pb, b);
    auto sw = [](const float* f) {
        Sweep s;
        s.localCenter = V(f[0], f[1]); s.c0 = V(f[2], f[3]); s.c = V(f[4], f[5]);
        s.a0 = f[6]; s.a = f[7]; s.alpha0 = f[8];
        return s;
    };
    int state;
    float t;
    TimeOfImpact(&state, &t, pa, pb, sw(swA), sw(swB), tMax);
    out[0] = (float)state;
    out[1] = t;
}

void po_sincosf(float x, float* s, float* c) { Rot q = RotOf(x); *s = q.s; *c = q.c; }

// Island structure of the next Solve without stepping: for every island in solve order, its contacts
// in solve order as (bodyA, bodyB, static flags). Used to study the Gauss-Seidel dependency chain.
int po_island_contacts(void* h, int* out, int cap)
{
    World* w = static_cast<World*>(h);
    int n = 0, island = 0;
    std::vector<char> bodySeen(w->bodies.size(), 0), contactSeen(w->contacts.size(), 0);
    std::vector<int> stack;
    for (int seed = w->bodyList; seed != kNull; seed = w->bodies[seed].next) {
        const Body& sb = w->bodies[seed];
        if (bodySeen[seed] || !sb.IsAwake() || !(sb.flags & kBActive) || sb.type == kStatic) continue;
        stack.assign(1, seed);
        bodySeen[seed] = 1;
        std::vector<int> statics;
        while (!stack.empty()) {
            int b = stack.back();
            stack.pop_back();
            if (w->bodies[b].type == kStatic) { statics.push_back(b); continue; }
            for (int e = w->bodies[b].contactList; e != kNull; e = w->contacts[e >> 1].eNext[e & 1]) {
                int c = e >> 1;
                const Contact& ct = w->contacts[c];
                if (contactSeen[c] || !(ct.flags & kCEnabled) || !(ct.flags & kCTouching)) continue;
                contactSeen[c] = 1;
                int bA = w->fixtures[ct.fA].body, bB = w->fixtures[ct.fB].body;
                if (n < cap) {
                    out[4 * n] = island; out[4 * n + 1] = bA; out[4 * n + 2] = bB;
                    out[4 * n + 3] = (w->bodies[bA].type == kStatic) | ((w->bodies[bB].type == kStatic) << 1) | (ct.m.pointCount << 2);
                }
                ++n;
                int other = w->EdgeOther(e);
                if (bodySeen[other]) continue;
                bodySeen[other] = 1;
                stack.push_back(other);
            }
        }
        for (int s : statics) bodySeen[s] = 0;
        ++island;
    }
    return n;
}

void po_step_many(void** hs, int n, float dt, int vi, int pi, int steps, int threads)
{
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([=]() {
            for (int i = t; i < n; i += threads)
                for (int s = 0; s < steps; ++s) static_cast<World*>(hs[i])->Step(dt, vi, pi);
        });
    }
    for (std::thread& th : pool) th.join();
}

} // extern "C"
