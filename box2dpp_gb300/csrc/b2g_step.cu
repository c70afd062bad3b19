// GB300 kernels for one Box2D 2.3.2 b2World::Step per world: contact update (narrowphase), island
// construction and solve, fixture synchronisation, broadphase pair finding and contact creation, and
// the continuous (time of impact) pass. One thread block (CTA) owns one world for the whole step;
// the order-defining parts (island DFS, contact creation, the TOI event loop) run on the CTA's first
// thread, everything else is spread across the CTA. The reference's results depend on the order of
// contacts inside islands and of contact creation, and that order is reproduced exactly.
//
// Built with -fmad=false (no contraction to FMA) and IEEE division/square root, so that the float
// arithmetic rounds as the reference does.
#include <cuda_runtime.h>

#include <climits>

#include "b2g_world.h"

namespace b2g {

// Walk a linked list with an iteration bound: a list longer than `lim` can only be corrupt, so the
// walk stops and flags the world instead of spinning.
#define B2G_WALK(e, head, next, lim)                                                                  \
    for (int e = (head), e##_n = 0; e != kNullIdx && (++e##_n <= (lim) || (atomicOr(&st->error, kErrInvalid), false)); \
         e = (next))

// ------------------------------------------------------------------ world view
struct Wd {
    WorldDesc d;
    WorldState* st;
    float4 *xf, *sw, *sw0, *vel, *frc, *mas, *prop;
    int4 *bi, *bj;
    int4* fi;
    float4* fm;
    int4* ff;
    float4* faabb;
    const Shape* shape;
    float4* fat;
    int* pfix;
    int* moved;
    int4 *ci, *ce;
    float4* cp;
    int4* mh;
    float4 *mv, *mp0, *mp1;
    int* order;      // the contact list: orderBase + st->orderStart
    int* orderBase;
    int* cnext;
    Joint* jt;
    int *sBody, *sStack, *sWake;
    float4 *sPos, *sVel;
    int *sContact, *sStatus;
    VelConstraint* vc;
    PosConstraint* pc;
    float4* vimp;
    float4* vimpL;
    float2* vsep;
    float4* sVelL;
    TOITask* toi;
    int4* islands;
    int2* islandJ;
    int* sJoint;
    int* sleepOut;
    int* cColour;
    int* colourList;
    int* evType;
    int4* evLog;
    int evCap;
    unsigned long long* rowMask;
    unsigned long long* pairs;
    int* pairKeep;
    int* movedList;
    int* liveProxies;
    int* gridIds;
    int* gridNext;
    int* gridPrev;
    int* gridCellOf;
    int* gridHead;
    int4* pairInfo;
    unsigned char* islTab; // the world's global island-table region (d.islTabBytes bytes)
    int wIndex;            // the world's index in the batch
    unsigned long long* filterKeys;  // user contact-filter verdicts (Batch::filterKeys), or nullptr
    int* filterVals;
    int filterCap;
    int* filterMiss;
    int filterMissCap;
    float4* smemBase;   // the CTA's dynamic shared memory, free outside the island solve
    int smemBytes;
    int* treeLogId;     // the world's tree-log records (Batch::treeLogId), or nullptr
    float4* treeLogFat;
    int treeLogCap;

    __device__ void init(const Batch& B, int w)
    {
        d = B.desc[w];
        st = B.state + w;
        int b = d.bodyBase, f = d.fixBase, p = d.proxyBase, c = d.contactBase, j = d.jointBase, q = d.pairBase;
        xf = B.xf + b; sw = B.sw + b; sw0 = B.sw0 + b; vel = B.vel + b; frc = B.frc + b; mas = B.mas + b;
        prop = B.prop + b; bi = B.bi + b; bj = B.bj + b;
        fi = B.fi + f; fm = B.fm + f; ff = B.ff + f; faabb = B.faabb + f; shape = B.shape + f;
        fat = B.fat + p; pfix = B.pfix + p; moved = B.moved + p; movedList = B.movedList + p; liveProxies = B.liveProxies + p;
        gridIds = B.gridIds + p; gridNext = B.gridNext + p; gridPrev = B.gridPrev + p; gridCellOf = B.gridCellOf + p;
        gridHead = B.gridHead + q + w;
        ci = B.ci + c; ce = B.ce + c; cp = B.cp + c; mh = B.mh + c; mv = B.mv + c; mp0 = B.mp0 + c; mp1 = B.mp1 + c;
        orderBase = B.order + 2 * (size_t)c;
        order = orderBase + st->orderStart;
        cnext = B.cnext + c;
        jt = B.joint + j; sJoint = B.sJoint + j;
        sBody = B.sBody + d.rowBase; sPos = B.sPos + d.rowBase; sVel = B.sVel + d.rowBase;
        rowMask = B.rowMask + d.rowBase; sVelL = B.sVelL + d.rowBase;
        sStack = B.sStack + b; sWake = B.sWake + b;
        islands = B.islands + b; islandJ = B.islandJ + b; sleepOut = B.sleepOut + b;
        sContact = B.sContact + c; sStatus = B.sStatus + c; vc = B.vc + c; pc = B.pc + c; vimp = B.vimp + c; toi = B.toi + c;
        vimpL = B.vimpL + c; vsep = B.vsep + c;
        cColour = B.cColour + c; colourList = B.colourList + c; evType = B.evType + c;
        evLog = B.evLog ? B.evLog + 8 * (size_t)c : nullptr;
        evCap = 4 * d.contactCap;
        pairs = B.pairs + q; pairKeep = B.pairKeep + q; pairInfo = B.pairInfo + q;
        islTab = B.islTab ? B.islTab + d.islTabBase : nullptr;
        wIndex = w;
        filterKeys = B.filterKeys;
        filterVals = B.filterVals;
        filterCap = B.filterCap;
        filterMiss = B.filterMiss;
        filterMissCap = B.filterMissCap;
        smemBase = nullptr;
        smemBytes = 0;
        if (B.treeLogId) {
            const size_t at = (size_t)kTreeLogPerProxy * d.proxyBase + (size_t)kTreeLogExtra * w;
            treeLogId = B.treeLogId + at;
            treeLogFat = B.treeLogFat + at;
            treeLogCap = kTreeLogPerProxy * d.proxyCap + kTreeLogExtra;
        } else {
            treeLogId = nullptr;
            treeLogFat = nullptr;
            treeLogCap = 0;
        }
    }

    // One tree-log record (a proxy's new fat box, or a step mark). Past the log's room the count still
    // grows, which tells the host that the tree's history is incomplete.
    __device__ void treeLog(int pid, float4 fat, int kind)
    {
        const int k = atomicAdd(&st->treeLogCount, 1);
        if (k >= treeLogCap) return;
        treeLogId[k] = pid << 2 | kind;
        treeLogFat[k] = fat;
    }

    // ---------------------------------------------------------------- listener event log
    __device__ void putEvent(int slot, int kind, int fA, int fB, int count = 0, float n0 = 0.0f, float n1 = 0.0f,
                             float t0 = 0.0f, float t1 = 0.0f)
    {
        if (slot >= evCap) { st->eventsDropped = 1; return; }
        evLog[2 * slot] = make_int4(kind, fA, fB, count);
        evLog[2 * slot + 1] = make_int4(__float_as_int(n0), __float_as_int(n1), __float_as_int(t0), __float_as_int(t1));
    }
    // the calls b2Contact::Update makes (Dynamics/Contacts/b2Contact.cpp:164-236), as bits: 1 begin,
    // 2 end, 4 pre-solve
    __device__ static int updateEventBits(bool wasTouching, bool touching, bool sensor)
    {
        return (!wasTouching && touching ? 1 : 0) | (wasTouching && !touching ? 2 : 0) | (!sensor && touching ? 4 : 0);
    }
    // serial append of a contact's update calls (one thread)
    __device__ void appendUpdateEvents(int c, int bits)
    {
        const int4 info = ci[c];
        for (int b = 0; b < 3; ++b)
            if (bits & (1 << b)) putEvent(st->eventCount++, b, info.y, info.z);
    }

    // ---------------------------------------------------------------- body helpers
    __device__ float4& vel_body(int b) { return vel[b]; }
    __device__ int type(int b) const { return bi[b].x; }
    __device__ int flags(int b) const { return bi[b].y; }
    __device__ bool awake(int b) const { return (bi[b].y & kBAwake) != 0; }
    __device__ Xf xform(int b) const
    {
        float4 t = xf[b];
        Xf x;
        x.p = V(t.x, t.y); x.q.s = t.z; x.q.c = t.w;
        return x;
    }
    __device__ void setXform(int b, const Xf& x) { xf[b] = make_float4(x.p.x, x.p.y, x.q.s, x.q.c); }
    __device__ Sweep sweep(int b) const
    {
        float4 a = sw[b], a0 = sw0[b], m = mas[b];
        Sweep s;
        s.localCenter = V(m.z, m.w);
        s.c0 = V(a0.x, a0.y); s.a0 = a0.z;
        s.c = V(a.x, a.y); s.a = a.z; s.alpha0 = a.w;
        return s;
    }
    __device__ void setSweep(int b, const Sweep& s)
    {
        sw[b] = make_float4(s.c.x, s.c.y, s.a, s.alpha0);
        float sleep = sw0[b].w;
        sw0[b] = make_float4(s.c0.x, s.c0.y, s.a0, sleep);
    }
    // b2Body::SetAwake (Dynamics/b2Body.h:625-645)
    __device__ void setAwake(int b, bool flag)
    {
        int fl = bi[b].y;
        if (flag) {
            if ((fl & kBAwake) == 0) {
                bi[b].y = fl | kBAwake;
                sw0[b].w = 0.0f;
            }
        } else {
            bi[b].y = fl & ~kBAwake;
            sw0[b].w = 0.0f;
            vel[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            frc[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    // b2Body::SynchronizeTransform (Dynamics/b2Body.h:850-854)
    __device__ void syncTransform(int b)
    {
        float4 a = sw[b], m = mas[b];
        Xf x;
        x.q = RotOf(a.z);
        x.p = V(a.x, a.y) - Mul(x.q, V(m.z, m.w));
        setXform(b, x);
    }
    // b2Body::Advance (Dynamics/b2Body.h:856-864)
    __device__ void advance(int b, float alpha)
    {
        Sweep s = sweep(b);
        SweepAdvance(s, alpha);
        s.c = s.c0;
        s.a = s.a0;
        setSweep(b, s);
        Xf x;
        x.q = RotOf(s.a);
        x.p = s.c - Mul(x.q, s.localCenter);
        setXform(b, x);
    }

    // ---------------------------------------------------------------- contact edge helpers
    // Edge e = 2*slot + side: side 0 is on bodyA's list (other = bodyB), side 1 on bodyB's list.
    __device__ int* ePrevP(int e) { return reinterpret_cast<int*>(&ce[e >> 1]) + ((e & 1) ? 2 : 0); }
    __device__ int* eNextP(int e) { return reinterpret_cast<int*>(&ce[e >> 1]) + ((e & 1) ? 3 : 1); }
    __device__ int eNext(int e) const
    {
        int4 v = ce[e >> 1];
        return (e & 1) ? v.w : v.y;
    }
    __device__ int fixBody(int f) const { return fi[f].x; }
    __device__ int edgeOther(int e) const
    {
        int4 c = ci[e >> 1];
        return (e & 1) == 0 ? fixBody(c.z) : fixBody(c.y);
    }
    __device__ int jNext(int e) const { return jt[e >> 1].eNext[e & 1]; }
    __device__ int jOther(int e) const { return (e & 1) == 0 ? jt[e >> 1].bodyB : jt[e >> 1].bodyA; }

    // b2Body::ShouldCollide (Dynamics/b2Body.cpp:354-375), called as bodyB->ShouldCollide(bodyA)
    __device__ bool shouldCollide(int self, int other) const
    {
        if (type(self) != kDynamic && type(other) != kDynamic) return false;
        B2G_WALK(e, bj[self].x, jNext(e), 2 * d.jointCount + 2)
            if (jOther(e) == other && !jt[e >> 1].collideConnected) return false;
        return true;
    }
    // default b2ContactFilter::ShouldCollide (Dynamics/b2WorldCallbacks.cpp:26-38)
    __device__ bool defaultFilter(int fA, int fB) const
    {
        int4 a = ff[fA], b = ff[fB];
        if (a.z == b.z && a.z != 0) return a.z > 0;
        return (a.y & b.x) != 0 && (a.x & b.y) != 0;
    }
    // b2ContactFilter::ShouldCollide as the world's filter decides it: the default filter, or the
    // user filter's verdict for this ordered fixture pair. A pair without a verdict yet is logged for
    // the host (which asks the user's filter after the step) and takes the default filter's verdict
    // for now; the host re-runs the step from its start when a logged verdict differs. The probe is
    // bounded by the table size; a full table is a capacity error.
    __device__ bool filterCollide(int fA, int fB) const
    {
        if (!filterKeys) return defaultFilter(fA, fB);
        const unsigned long long key = FilterKey(wIndex, fA, fB);
        unsigned slot = FilterSlot(key, filterCap);
        for (int probe = 0; probe < filterCap; ++probe, slot = (slot + 1) & (unsigned)(filterCap - 1)) {
            unsigned long long k = filterKeys[slot];
            if (k == ~0ull) {
                k = atomicCAS(&filterKeys[slot], ~0ull, key);
                if (k == ~0ull) {
                    const int m = atomicAdd(&filterMiss[0], 1);
                    if (m < filterMissCap) {
                        filterMiss[1 + 3 * m] = wIndex;
                        filterMiss[2 + 3 * m] = fA;
                        filterMiss[3 + 3 * m] = fB;
                    }
                    return defaultFilter(fA, fB);
                }
            }
            if (k == key) {
                const int v = filterVals[slot];
                return v == 2 ? defaultFilter(fA, fB) : v != 0;
            }
        }
        atomicOr(&st->error, kErrCapacity);
        return defaultFilter(fA, fB);
    }

    // ---------------------------------------------------------------- manifold IO
    __device__ void loadManifold(int c, Manifold& m) const
    {
        int4 h = mh[c];
        float4 v = mv[c], p0 = mp0[c], p1 = mp1[c];
        m.type = h.x; m.count = h.y;
        m.p[0].id = (uint32_t)h.z; m.p[1].id = (uint32_t)h.w;
        m.localNormal = V(v.x, v.y); m.localPoint = V(v.z, v.w);
        m.p[0].lp = V(p0.x, p0.y); m.p[0].ni = p0.z; m.p[0].ti = p0.w;
        m.p[1].lp = V(p1.x, p1.y); m.p[1].ni = p1.z; m.p[1].ti = p1.w;
    }
    __device__ void storeManifold(int c, const Manifold& m)
    {
        mh[c] = make_int4(m.type, m.count, (int)m.p[0].id, (int)m.p[1].id);
        mv[c] = make_float4(m.localNormal.x, m.localNormal.y, m.localPoint.x, m.localPoint.y);
        mp0[c] = make_float4(m.p[0].lp.x, m.p[0].lp.y, m.p[0].ni, m.p[0].ti);
        mp1[c] = make_float4(m.p[1].lp.x, m.p[1].lp.y, m.p[1].ni, m.p[1].ti);
    }

    // Copies the shape of fixture f to dst, 8 bytes at a time (shapes are 8-byte aligned).
    __device__ void stageShape(int f, Shape* dst) const
    {
        static_assert(sizeof(Shape) % 8 == 0, "shapes are copied as float2");
        const float2* src = reinterpret_cast<const float2*>(shape + f);
        float2* out = reinterpret_cast<float2*>(dst);
#pragma unroll
        for (int k = 0; k < (int)(sizeof(Shape) / 8); ++k) out[k] = src[k];
    }

    // b2Contact::Update's evaluation of a non-sensor contact (Dynamics/Contacts/b2Contact.cpp:176-209):
    // the manifold at the bodies' current transforms, each new point taking the impulses of the old
    // point with the same id. stage (optional): this thread's two shape slots in shared memory; the
    // narrowphase then reads both shapes there instead of re-reading them from global memory.
    __device__ void evaluateManifold(int c, Manifold& m, Shape* stage) const
    {
        const int4 info = ci[c];
        const int fA = info.y, fB = info.z;
        const Xf xfA = xform(fixBody(fA)), xfB = xform(fixBody(fB));
        Manifold old;
        loadManifold(c, old);
        m.count = 0;
        m.type = old.type;
        m.localNormal = old.localNormal;
        m.localPoint = old.localPoint;
        if (stage) {
            stageShape(fA, stage);
            stageShape(fB, stage + 1);
            Evaluate(&m, stage[0], xfA, stage[1], xfB);
        } else {
            Evaluate(&m, shape[fA], xfA, shape[fB], xfB);
        }
        for (int i = 0; i < m.count; ++i) {
            m.p[i].ni = 0.0f;
            m.p[i].ti = 0.0f;
            for (int j = 0; j < old.count; ++j) {
                if (old.p[j].id == m.p[i].id) {
                    m.p[i].ni = old.p[j].ni;
                    m.p[i].ti = old.p[j].ti;
                    break;
                }
            }
        }
        for (int i = m.count; i < 2; ++i) { m.p[i].lp = V(0.0f, 0.0f); m.p[i].ni = 0.0f; m.p[i].ti = 0.0f; m.p[i].id = 0; }
    }

    // Stage record of contact c (see ManifoldStage; it shares the contact's VelConstraint slot).
    __device__ ManifoldStage* stageOf(int c) const { return reinterpret_cast<ManifoldStage*>(vc) + c; }
    __device__ void writeStage(int c, const Manifold& m) const
    {
        ManifoldStage* S = stageOf(c);
        S->h = make_int4(m.type, m.count, (int)m.p[0].id, (int)m.p[1].id);
        S->v = make_float4(m.localNormal.x, m.localNormal.y, m.localPoint.x, m.localPoint.y);
        S->p0 = make_float4(m.p[0].lp.x, m.p[0].lp.y, m.p[0].ni, m.p[0].ti);
        S->p1 = make_float4(m.p[1].lp.x, m.p[1].lp.y, m.p[1].ni, m.p[1].ti);
    }

    // b2Contact::Update (Dynamics/Contacts/b2Contact.cpp:164-245). Returns true when the touching
    // state of a non-sensor contact changed (the caller wakes both bodies). staged: this step's
    // NarrowphaseKernel ran for the world, so a contact it evaluated (tag 1) commits that record,
    // the same values the evaluation here would give.
    __device__ bool update(int c, Shape* stage = nullptr, bool staged = false)
    {
        int4 info = ci[c];
        int fl = info.x | kCEnabled;
        bool wasTouching = (fl & kCTouching) != 0;
        int fA = info.y, fB = info.z;
        bool sensor = fi[fA].w != 0 || fi[fB].w != 0;
        bool touching;
        bool changed = false;
        if (sensor) {
            int bA = fixBody(fA), bB = fixBody(fB);
            Xf xfA = xform(bA), xfB = xform(bB);
            Proxy pa = ProxyOf(shape[fA]), pb = ProxyOf(shape[fB]);
            SimplexCache cache;
            cache.count = 0;
            cache.metric = 0.0f;
            Vec2 a, b;
            touching = Distance(&a, &b, &cache, pa, xfA, pb, xfB, true) < 10.0f * kEpsilon;
            mh[c].y = 0;
        } else {
            const ManifoldStage* S = stageOf(c);
            if (staged && S->tag == 1) {
                const int4 h = S->h;
                mh[c] = h;
                mv[c] = S->v;
                mp0[c] = S->p0;
                mp1[c] = S->p1;
                touching = h.y > 0;
            } else {
                Manifold m;
                evaluateManifold(c, m, stage);
                storeManifold(c, m);
                touching = m.count > 0;
            }
            changed = touching != wasTouching;
        }
        if (touching) fl |= kCTouching;
        else fl &= ~kCTouching;
        ci[c].x = fl;
        return changed;
    }

    // ---------------------------------------------------------------- broadphase
    // b2Fixture::Synchronize + b2DynamicTree::MoveProxy (b2Fixture.cpp:154-177, b2DynamicTree.cpp:133-177)
    // movedOut (optional, one thread): the proxies this call marks moved are appended to movedList
    __device__ void syncFixtures(int b, int* movedOut = nullptr, int logKind = kTreeOrdered)
    {
        float4 s0 = sw0[b], m = mas[b];
        Xf xf1;
        xf1.q = RotOf(s0.z);
        xf1.p = V(s0.x, s0.y) - Mul(xf1.q, V(m.z, m.w));
        syncFixturesFrom(b, xf1, xform(b), movedOut, logKind);
    }

    // b2Fixture::Synchronize (Dynamics/b2Fixture.cpp:154-177) of every fixture of body b between two
    // transforms, with b2BroadPhase::MoveProxy (b2DynamicTree.cpp:133-177): the swept AABB, and a
    // new fat AABB (grown by the extension and the predicted displacement) when it left the old one.
    // logKind: the tree-log kind of the re-insertions (when the world keeps a tree log).
    __device__ void syncFixturesFrom(int b, const Xf& xf1, const Xf& xf2, int* movedOut = nullptr,
                                     int logKind = kTreeOrdered)
    {
        B2G_WALK(f, bi[b].z, fi[f].y, d.fixCount + 1) {
            int pid = fi[f].z;
            if (pid < 0) continue;
            const Shape& sh = shape[f];
            float4 a = Combine(ComputeAABB(sh, xf1), ComputeAABB(sh, xf2));
            faabb[f] = a;
            Vec2 disp = xf2.p - xf1.p;
            if (Contains(fat[pid], a)) continue;
            float4 nb;
            nb.x = a.x - kAabbExtension; nb.y = a.y - kAabbExtension;
            nb.z = a.z + kAabbExtension; nb.w = a.w + kAabbExtension;
            Vec2 dd = kAabbMultiplier * disp;
            if (dd.x < 0.0f) nb.x += dd.x; else nb.z += dd.x;
            if (dd.y < 0.0f) nb.y += dd.y; else nb.w += dd.y;
            fat[pid] = nb;
            if (treeLogId) treeLog(pid, nb, logKind);
            if (movedOut && moved[pid] == 0) movedList[(*movedOut)++] = pid;
            moved[pid] = 1;
        }
    }

    // One b2Body state change between steps (the methods gb_body_edits lists, Dynamics/b2Body.cpp:
    // 419-441 and b2Body.h:501-830), with the reference's type checks, wakes and sleep rules.
    __device__ void applyEdit(const BodyEdit& e)
    {
        if (e.op == kEditMouseTarget) {
            // b2MouseJoint::SetTarget (Dynamics/Joints/b2MouseJoint.cpp:54-61): wakes body B
            Joint& J = jt[e.body];
            if (!awake(J.bodyB)) setAwake(J.bodyB, true);
            J.target = V(e.v[0], e.v[1]);
            return;
        }
        const int b = e.body;
        const int type = bi[b].x;
        auto wakeOnRequest = [&]() {
            if (e.wake && !awake(b)) setAwake(b, true);
        };
        switch (e.op) {
        case kEditSetTransform: {
            Xf x;
            x.q = RotOf(e.v[2]);
            x.p = V(e.v[0], e.v[1]);
            const float4 m = mas[b];
            const Vec2 c = Mul(x, V(m.z, m.w));
            setXform(b, x);
            sw[b] = make_float4(c.x, c.y, e.v[2], sw[b].w);
            sw0[b] = make_float4(c.x, c.y, e.v[2], sw0[b].w);
            syncFixturesFrom(b, x, x);
            break;
        }
        case kEditSetLinearVelocity: {
            if (type == kStatic) break;
            const Vec2 v = V(e.v[0], e.v[1]);
            if (Dot(v, v) > 0.0f) setAwake(b, true);
            float4 q = vel[b];
            q.x = v.x;
            q.y = v.y;
            vel[b] = q;
            break;
        }
        case kEditSetAngularVelocity:
            if (type == kStatic) break;
            if (e.v[0] * e.v[0] > 0.0f) setAwake(b, true);
            vel[b].z = e.v[0];
            break;
        case kEditSetAwake:
            setAwake(b, e.v[0] != 0.0f);
            break;
        case kEditApplyForce:
        case kEditApplyForceToCenter:
        case kEditApplyTorque: {
            if (type != kDynamic) break;
            wakeOnRequest();
            if (!awake(b)) break;
            float4 f = frc[b];
            if (e.op == kEditApplyTorque) {
                f.z += e.v[0];
            } else {
                f.x += e.v[0];
                f.y += e.v[1];
                if (e.op == kEditApplyForce) {
                    const float4 s = sw[b];
                    f.z += Cross(V(e.v[2], e.v[3]) - V(s.x, s.y), V(e.v[0], e.v[1]));
                }
            }
            frc[b] = f;
            break;
        }
        case kEditApplyLinearImpulse:
        case kEditApplyAngularImpulse: {
            if (type != kDynamic) break;
            wakeOnRequest();
            if (!awake(b)) break;
            const float4 m = mas[b];
            float4 q = vel[b];
            if (e.op == kEditApplyLinearImpulse) {
                const float4 s = sw[b];
                q.x += m.x * e.v[0];
                q.y += m.x * e.v[1];
                q.z += m.y * Cross(V(e.v[2], e.v[3]) - V(s.x, s.y), V(e.v[0], e.v[1]));
            } else {
                q.z += m.y * e.v[0];
            }
            vel[b] = q;
            break;
        }
        default:
            break;
        }
    }

    // Contact factory order (Dynamics/Contacts/b2Contact.cpp:40-100): primary type pairs keep (A, B).
    __device__ static bool primaryOrder(int t1, int t2) { return t1 == t2 || (t1 == kPolygon && t2 == kCircle) || t1 == kEdge; }

    // b2ContactManager::FindNewContacts -> b2BroadPhase::UpdatePairs -> AddPair, CTA-wide.
    __device__ void findNewContacts(bool inToi = false, int knownMoved = -1);
    __device__ void gridPairs(int m, int* pairCount);
    __device__ void gridEventPairs(int m, int* pairCount);
    __device__ void collide();
    __device__ void solve(const StepParams& P, float4* smem, int smemRows, int smemContacts);
    template <class L>
    __device__ bool buildIslandsTable(unsigned char* base, int capacity, bool coloured, int* colourCount, int& nIsl,
                                      int& nRows, int& nCons, int& movers);
    template <class L>
    __device__ bool buildIslandsParallel(unsigned char* base, int capacity, int* radixWork, int* colourCount, int& nIsl,
                                         int& nRows, int& nCons, int& movers);
    __device__ void solveIslands(const StepParams& P, int nIsl, int nRows, int nContacts, float4* smem, int smemRows,
                                 int smemContacts, const int* colourStart);
    __device__ void solveTOI(const StepParams& P);
    __device__ void resetToi();
    __device__ int toiKind(const int4& info) const;
    __device__ void warmStartAll(int nIsl, const int* colourStart, const float4* im, float4* v);
    __device__ void learnedImpulses(const StepParams& P, int nContacts, const float4* imp, const float4* vel);
    __device__ void destroyContact(int c);
};

// ------------------------------------------------------------------ CTA helpers
__device__ inline int tid() { return threadIdx.x; }
__device__ inline int nthreads() { return blockDim.x; }

// Appends to a list counted by *count (shared memory) with one atomic per warp: returns this lane's
// slot when keep, else -1. Every lane of the warp must call it (CTA sizes are multiples of 32).
__device__ inline int WarpAppend(bool keep, int* count)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    int base = 0;
    if (lane == 0 && bal) base = atomicAdd(count, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    return keep ? base + __popc(bal & ((1u << lane) - 1u)) : -1;
}

// Largest CTA of a per-world launch.
constexpr int kMaxCta = 512;
// the continuous phase (StepToiKernel) runs with at most this many threads per CTA
// the continuous phase's CTA width: its event loop is one thread's work, so in a batch narrower CTAs
// let more worlds' loops run side by side (bench batch, one call: 3.49 ms per step at 128 threads,
// 3.40 at 64, 3.55 at 32); a class of one world keeps the wider CTA (kMaxToiCta, which also sizes the
// loop's shared arrays)
constexpr int kMaxToiCta = 128;
constexpr int kBatchToiCta = 64;

// Exclusive prefix sums over the CTA of up to three per-thread counts (threads in index order), by
// warp shuffles and one shared slot per warp and count; totals receive the CTA-wide sums. Every
// thread of the CTA calls it (CTA sizes are multiples of 32).
__device__ inline void ctaExclusiveScan3(int& a, int& b, int& c, int* totals)
{
    __shared__ int sWarp[3][kMaxCta / 32 + 1];
    const int lane = tid() & 31, warp = tid() >> 5, nWarps = (nthreads() + 31) >> 5;
    int ia = a, ib = b, ic = c;
    for (int o = 1; o < 32; o <<= 1) {
        const int xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o),
                  xc = __shfl_up_sync(0xffffffffu, ic, o);
        if (lane >= o) { ia += xa; ib += xb; ic += xc; }
    }
    if (lane == 31) { sWarp[0][warp] = ia; sWarp[1][warp] = ib; sWarp[2][warp] = ic; }
    __syncthreads();
    int pa = 0, pb = 0, pc = 0, ta = 0, tb = 0, tc = 0;
    for (int w = 0; w < nWarps; ++w) {
        if (w < warp) { pa += sWarp[0][w]; pb += sWarp[1][w]; pc += sWarp[2][w]; }
        ta += sWarp[0][w]; tb += sWarp[1][w]; tc += sWarp[2][w];
    }
    a = pa + ia - a;
    b = pb + ib - b;
    c = pc + ic - c;
    totals[0] = ta;
    totals[1] = tb;
    totals[2] = tc;
    __syncthreads();
}

// Order-preserving compaction over the CTA: out receives in[k] for every k < n with keep(k), in k
// order; returns the count (same value in every thread). Each thread takes one contiguous chunk.
template <typename Keep>
__device__ int ctaCompact(const int* in, int n, int* out, Keep keep)
{
    const int T = nthreads(), t = tid();
    const int chunk = (n + T - 1) / T;
    const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
    int o = 0, u1 = 0, u2 = 0, tot[3];
    for (int k = lo; k < hi; ++k) o += keep(k) ? 1 : 0;
    ctaExclusiveScan3(o, u1, u2, tot);
    for (int k = lo; k < hi; ++k)
        if (keep(k)) out[o++] = in[k];
    __syncthreads();
    return tot[0];
}

// Bitonic sort of n 64-bit keys in global memory (n <= capacity, capacity a power of two); the
// padding keys are all-ones so they sort last.
__device__ void ctaSortKeys(unsigned long long* keys, int n, int capacity)
{
    int P = 1;
    while (P < n) P <<= 1;
    if (P > capacity) P = capacity;
    for (int i = n + tid(); i < P; i += nthreads()) keys[i] = ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid(); i < P; i += nthreads()) {
                int l = i ^ j;
                if (l > i) {
                    unsigned long long a = keys[i], b = keys[l];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) { keys[i] = b; keys[l] = a; }
                }
            }
            __syncthreads();
        }
    }
}

// Stable LSD radix sort (8-bit digits) of n 64-bit keys in global memory over the CTA, ping-ponging
// between keys and tmp (n slots each); the sorted keys end in keys. A digit position where every key
// has the same byte is skipped (its pass would not move anything). For arrays too large for shared
// memory this replaces the bitonic network, whose log^2 n passes over global memory dominate large
// worlds; both give the same order (equal keys are equal values). work: kRadixWork ints of shared
// memory (the digit bases and the per-warp tile counts); the caller checks RadixSortFits first.
constexpr int kRadixWork = 256 + (kMaxCta / 32) * 256;
// the work a CTA of this launch uses: the digit bases and one row of tile counts per warp
__device__ inline int RadixWorkInts() { return 256 + ((nthreads() + 31) / 32) * 256; }
__device__ inline bool RadixSortFits(int n, int workBytes)
{
    // tile stamps are packed with a 6-bit count into an int: at most 2^24 tiles over all passes
    return workBytes >= RadixWorkInts() * (int)sizeof(int) && (long long)((n + 31) / 32) * 8 < (1ll << 24);
}
__device__ void ctaRadixSort(unsigned long long* keys, unsigned long long* tmp, int n, int* work)
{
    __shared__ unsigned long long sOr, sAnd;
    int* sBase = work;
    int (*sTileCnt)[256] = reinterpret_cast<int (*)[256]>(work + 256);
    if (n <= 1) return;
    const int T = nthreads(), t = tid(), lane = t & 31, warp = t >> 5;
    if (t == 0) { sOr = 0ull; sAnd = ~0ull; }
    for (int i = t; i < ((T + 31) / 32) * 256; i += T) work[256 + i] = -1;
    __syncthreads();
    {
        unsigned long long o = 0ull, a = ~0ull;
        for (int i = t; i < n; i += T) { o |= keys[i]; a &= keys[i]; }
        atomicOr(&sOr, o);
        atomicAnd(&sAnd, a);
    }
    __syncthreads();
    const unsigned long long varying = sOr ^ sAnd;
    const int nTiles = (n + T - 1) / T;
    unsigned long long* src = keys;
    unsigned long long* dst = tmp;
    int stampBase = 0;
    for (int shift = 0; shift < 64; shift += 8) {
        if (((varying >> shift) & 0xffull) == 0ull) continue;
        for (int dg = t; dg < 256; dg += T) sBase[dg] = 0;
        __syncthreads();
        for (int i = t; i < n; i += T) atomicAdd(&sBase[(int)((src[i] >> shift) & 0xffull)], 1);
        __syncthreads();
        if (t == 0) {
            int run = 0;
            for (int dg = 0; dg < 256; ++dg) { const int c = sBase[dg]; sBase[dg] = run; run += c; }
        }
        __syncthreads();
        // tiles of T consecutive keys: a key's place is its digit's base, plus the keys with the same
        // digit in earlier warps of the tile (sTileCnt, stamped with the tile), plus its rank in its
        // warp (lanes in index order), which keeps the pass stable
        for (int tile = 0; tile < nTiles; ++tile) {
            const int i = tile * T + t;
            const bool valid = i < n;
            const unsigned long long key = valid ? src[i] : 0ull;
            const int dg = valid ? (int)((key >> shift) & 0xffull) : 256;
            const unsigned peers = __match_any_sync(0xffffffffu, dg);
            const int rank = __popc(peers & ((1u << lane) - 1u));
            const bool leader = rank == 0;
            const int cnt = __popc(peers);
            const int stamp = stampBase + tile;
            if (valid && leader) sTileCnt[warp][dg] = (stamp << 6) | cnt;
            __syncthreads();
            if (valid) {
                int off = 0;
                for (int w2 = 0; w2 < warp; ++w2) {
                    const int v = sTileCnt[w2][dg];
                    if ((v >> 6) == stamp) off += v & 63;
                }
                dst[sBase[dg] + off + rank] = key;
            }
            __syncthreads();
            if (valid && leader) atomicAdd(&sBase[dg], cnt);
            __syncthreads();
        }
        stampBase += nTiles;
        unsigned long long* x = src;
        src = dst;
        dst = x;
    }
    if (src != keys) {
        for (int i = t; i < n; i += T) keys[i] = src[i];
        __syncthreads();
    }
}

// ------------------------------------------------------------------ FindNewContacts
// Above this many moved x live proxy tests, pair finding bins the proxies into a grid instead.
constexpr long long kSweepThreshold = 1ll << 20;

__device__ inline unsigned OrderedBits(float x)
{
    const unsigned u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ inline float FromOrderedBits(unsigned o)
{
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// The pairs of b2BroadPhase::UpdatePairs for large worlds, the same set the all-pairs test finds
// (the overlap test is b2TestOverlap, only the candidates differ): live proxies are binned by the
// lower corner of their fat AABB into a uniform grid whose cells are at least as wide and as tall as
// the largest proxy, and sorted by cell; each moved proxy tests the proxies of the cells that its box,
// grown by that size down and left, covers. A proxy overlapping it has its lower corner in that grown
// box, and the cell of a coordinate, floor((x - origin) / h), never decreases with x, so those cells
// hold every candidate. Proxies more than 4x larger than the mean (container edges, ground) stay out
// of the grid and are tested against every moved proxy. Keys live in the pair-info scratch (free
// until contact creation), the cell ranges after them.
__device__ void Wd::gridPairs(int m, int* pairCount)
{
    // moved proxies larger than the cell size (container walls, ground) are tested against every
    // live proxy with the scan spread over the CTA, one such proxy at a time, after the others
    constexpr int kLargeCap = 64;
    __shared__ int sLargeMoved[kLargeCap];
    __shared__ int sNLarge;
    __shared__ float sSizeSum;
    __shared__ int sLive, sSmall, sCursor;
    __shared__ unsigned sMaxW, sMinX, sMinY, sMaxX, sMaxY;
    const int np = d.proxyCap;
    if (tid() == 0) {
        sSizeSum = 0.0f; sLive = 0; sSmall = 0; sCursor = 0; sMaxW = 0u;
        sMinX = sMinY = 0xffffffffu; sMaxX = sMaxY = 0u;
        sNLarge = 0;
    }
    __syncthreads();
    auto size = [](const float4& f) { return fmaxf(f.z - f.x, f.w - f.y); };
    {
        float wsum = 0.0f;
        int live = 0;
        for (int p = tid(); p < np; p += nthreads())
            if (pfix[p] >= 0) { wsum += size(fat[p]); ++live; }
        atomicAdd(&sSizeSum, wsum);
        atomicAdd(&sLive, live);
    }
    __syncthreads();
    const int nLive = sLive;
    const float wLarge = 4.0f * (sSizeSum / (float)max(nLive, 1));
    {
        // extents of the small proxies: per thread, then per warp, then one atomic per warp
        unsigned maxW = 0u, minX = 0xffffffffu, minY = 0xffffffffu, maxX = 0u, maxY = 0u;
        for (int p0 = 0; p0 < np; p0 += nthreads()) {
            const int p = p0 + tid();
            if (p >= np || pfix[p] < 0) continue;
            const float4 f = fat[p];
            if (size(f) > wLarge) continue;
            maxW = max(maxW, __float_as_uint(fmaxf(size(f), 0.0f)));
            minX = min(minX, OrderedBits(f.x));
            minY = min(minY, OrderedBits(f.y));
            maxX = max(maxX, OrderedBits(f.x));
            maxY = max(maxY, OrderedBits(f.y));
        }
        maxW = __reduce_max_sync(0xffffffffu, maxW);
        minX = __reduce_min_sync(0xffffffffu, minX);
        minY = __reduce_min_sync(0xffffffffu, minY);
        maxX = __reduce_max_sync(0xffffffffu, maxX);
        maxY = __reduce_max_sync(0xffffffffu, maxY);
        if ((tid() & 31) == 0) {
            atomicMax(&sMaxW, maxW);
            atomicMin(&sMinX, minX);
            atomicMin(&sMinY, minY);
            atomicMax(&sMaxX, maxX);
            atomicMax(&sMaxY, maxY);
        }
    }
    __syncthreads();
    // the grid: cell size h >= the largest small proxy, at most cellCap cells (h grows to fit)
    const float W = __uint_as_float(sMaxW) * 1.0001f + 1e-4f;
    const bool anySmall = sMinX <= sMaxX;
    const float ox = anySmall ? FromOrderedBits(sMinX) : 0.0f, oy = anySmall ? FromOrderedBits(sMinY) : 0.0f;
    float spanX = anySmall ? FromOrderedBits(sMaxX) - ox : 0.0f;
    float spanY = anySmall ? FromOrderedBits(sMaxY) - oy : 0.0f;
    if (!(spanX < 1e30f) || !(spanY < 1e30f)) spanX = spanY = 0.0f;  // non-finite boxes: one cell (all-pairs)
    const int cellCap = min(d.pairCap, 4 * max(nLive, 1));
    float h = fmaxf(W, 1e-3f), invH, fx, fy;
    for (;;) {
        invH = 1.0f / h;
        fx = floorf(spanX * invH) + 1.0f;
        fy = floorf(spanY * invH) + 1.0f;
        if (fx * fy <= (float)cellCap) break;
        h *= 1.5f;
    }
    const int nx = (int)fx, ny = (int)fy;
    auto cellOf = [&](float x, float o, int n) {
        const float c = fminf(fmaxf(floorf((x - o) * invH), -1.0f), (float)n);
        return (int)c;
    };
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(pairInfo);
    // keys: cell << 32 | proxy for the small proxies, all-ones << 32 | proxy for the large ones, so
    // they sort last
    {
        int small = 0;
        for (int p0 = 0; p0 < np; p0 += nthreads()) {
            const int p = p0 + tid();
            const bool live = p < np && pfix[p] >= 0;
            unsigned hi = 0xffffffffu;
            if (live) {
                const float4 f = fat[p];
                if (!(size(f) > wLarge)) {
                    const int cx = min(max(cellOf(f.x, ox, nx), 0), nx - 1), cy = min(max(cellOf(f.y, oy, ny), 0), ny - 1);
                    hi = (unsigned)(cy * nx + cx);
                    ++small;
                }
            }
            const int slot = WarpAppend(live, &sCursor);
            if (slot >= 0) keys[slot] = ((unsigned long long)hi << 32) | (unsigned)p;
        }
        atomicAdd(&sSmall, small);
    }
    __syncthreads();
    int P2 = 1;
    while (P2 < nLive) P2 <<= 1;
    if (P2 * (int)sizeof(unsigned long long) <= smemBytes) {
        unsigned long long* sk = reinterpret_cast<unsigned long long*>(smemBase);
        for (int i = tid(); i < nLive; i += nthreads()) sk[i] = keys[i];
        __syncthreads();
        ctaSortKeys(sk, nLive, P2);
        for (int i = tid(); i < nLive; i += nthreads()) keys[i] = sk[i];
        __syncthreads();
    } else if (RadixSortFits(nLive, smemBytes)) {
        // the second half of the pair-info scratch (2 x pairCap keys, nLive <= pairCap) as the buffer
        ctaRadixSort(keys, keys + d.pairCap, nLive, reinterpret_cast<int*>(smemBase));
    } else {
        ctaSortKeys(keys, nLive, 2 * d.pairCap);
    }
    // cell ranges [start, end) in the second half of the scratch (2 x pairCap ints >= 2 x cellCap)
    const int nSmall = sSmall, nCells = nx * ny;
    int* cellStart = reinterpret_cast<int*>(keys + d.pairCap);
    int* cellEnd = cellStart + nCells;
    for (int c = tid(); c < nCells; c += nthreads()) { cellStart[c] = 0; cellEnd[c] = 0; }
    __syncthreads();
    for (int i = tid(); i < nSmall; i += nthreads()) {
        const unsigned c = (unsigned)(keys[i] >> 32);
        if (i == 0 || (unsigned)(keys[i - 1] >> 32) != c) cellStart[c] = i;
        if (i == nSmall - 1 || (unsigned)(keys[i + 1] >> 32) != c) cellEnd[c] = i + 1;
    }
    __syncthreads();
    // the grid kept for the continuous phase's events: each cell (and the large proxies, list nCells)
    // as a doubly linked list in the sorted order
    for (int i = tid(); i < nLive; i += nthreads()) {
        const unsigned long long k = keys[i];
        const int p = (int)(k & 0xffffffffu);
        const bool small = i < nSmall;
        const int c = small ? (int)(k >> 32) : nCells;
        const int lo = small ? cellStart[c] : nSmall, hi = small ? cellEnd[c] : nLive;
        gridIds[i] = p;
        gridPrev[p] = i > lo ? (int)(keys[i - 1] & 0xffffffffu) : -1;
        gridNext[p] = i + 1 < hi ? (int)(keys[i + 1] & 0xffffffffu) : -1;
        gridCellOf[p] = c;
    }
    for (int c = tid(); c <= nCells; c += nthreads()) {
        if (c < nCells) gridHead[c] = cellEnd[c] > cellStart[c] ? (int)(keys[cellStart[c]] & 0xffffffffu) : -1;
        else gridHead[c] = nLive > nSmall ? (int)(keys[nSmall] & 0xffffffffu) : -1;
    }
    if (tid() == 0) {
        st->gridValid = 1;
        st->gridNx = nx;
        st->gridNy = ny;
        st->gridLive = nLive;
        st->gridOx = ox;
        st->gridOy = oy;
        st->gridInvH = invH;
        st->gridW = W;
        st->gridWLarge = wLarge;
    }
    auto test = [&](int p, int q, const float4& Fq) {
        if (p == q) return;
        if (moved[p] && p < q) return;
        if (!Overlap(fat[p], Fq)) return;
        const int k = atomicAdd(pairCount, 1);
        const unsigned long long lo = (unsigned long long)(p < q ? p : q), hi = (unsigned long long)(p < q ? q : p);
        if (k < d.pairCap) pairs[k] = (lo << 32) | hi;
    };
    for (int t = tid(); t < m; t += nthreads()) {
        const int q = movedList[t];
        const float4 Fq = fat[q];
        if (size(Fq) > wLarge) {
            const int slot = atomicAdd(&sNLarge, 1);
            if (slot < kLargeCap) {
                sLargeMoved[slot] = q;
            } else {
                for (int j = 0; j < nLive; ++j) test((int)(keys[j] & 0xffffffffu), q, Fq);
            }
            continue;
        }
        const float lowX = Fq.x - W - 1e-4f * fabsf(Fq.x), lowY = Fq.y - W - 1e-4f * fabsf(Fq.y);
        const int cx0 = max(cellOf(lowX, ox, nx), 0), cx1 = min(cellOf(Fq.z, ox, nx), nx - 1);
        const int cy0 = max(cellOf(lowY, oy, ny), 0), cy1 = min(cellOf(Fq.w, oy, ny), ny - 1);
        for (int cy = cy0; cy <= cy1; ++cy)
            for (int cx = cx0; cx <= cx1; ++cx) {
                const int c = cy * nx + cx;
                for (int i = cellStart[c], e = cellEnd[c]; i < e; ++i) test((int)(keys[i] & 0xffffffffu), q, Fq);
            }
        for (int j = nSmall; j < nLive; ++j) test((int)(keys[j] & 0xffffffffu), q, Fq);
    }
    __syncthreads();
    const int nLarge = min(sNLarge, kLargeCap);
    for (int l = 0; l < nLarge; ++l) {
        const int q = sLargeMoved[l];
        const float4 Fq = fat[q];
        for (int j = tid(); j < nLive; j += nthreads()) test((int)(keys[j] & 0xffffffffu), q, Fq);
    }
    __syncthreads();
}

// The pairs of a continuous-phase event's moved proxies from the grid the step's pair finding kept:
// thread 0 moves each moved proxy to the cell list of its current box (so every live proxy sits in
// the list of its current low corner, or in the large proxies' list), then each moved proxy walks
// the lists of the cells its box can reach. Every live proxy is in exactly one list, so a pair is
// met once (both moved: from the lower id, as in the other paths).
__device__ void Wd::gridEventPairs(int m, int* pairCount)
{
    constexpr int kLargeCap = 64;
    __shared__ int sLargeQ[kLargeCap];
    __shared__ int sNLargeQ;
    const int nx = st->gridNx, ny = st->gridNy, nCells = nx * ny, nLive = st->gridLive;
    const float ox = st->gridOx, oy = st->gridOy, invH = st->gridInvH, wLarge = st->gridWLarge;
    auto size = [](const float4& f) { return fmaxf(f.z - f.x, f.w - f.y); };
    auto cellOf = [&](float x, float o, int n) {
        const float c = fminf(fmaxf(floorf((x - o) * invH), -1.0f), (float)n);
        return (int)c;
    };
    if (tid() == 0) {
        float W = st->gridW;
        for (int t = 0; t < m; ++t) {
            const int q = movedList[t];
            const float4 f = fat[q];
            int c = nCells;
            if (!(size(f) > wLarge)) {
                c = min(max(cellOf(f.y, oy, ny), 0), ny - 1) * nx + min(max(cellOf(f.x, ox, nx), 0), nx - 1);
                W = fmaxf(W, fmaxf(size(f), 0.0f) * 1.0001f + 1e-4f);
            }
            const int old = gridCellOf[q];
            if (old == c) continue;
            const int pv = gridPrev[q], nt = gridNext[q];
            if (pv >= 0) gridNext[pv] = nt;
            else gridHead[old] = nt;
            if (nt >= 0) gridPrev[nt] = pv;
            const int h = gridHead[c];
            gridPrev[q] = -1;
            gridNext[q] = h;
            if (h >= 0) gridPrev[h] = q;
            gridHead[c] = q;
            gridCellOf[q] = c;
        }
        st->gridW = W;
        sNLargeQ = 0;
    }
    __syncthreads();
    const float W = st->gridW;
    auto test = [&](int p, int q, const float4& Fq) {
        if (p == q) return;
        if (moved[p] && p < q) return;
        if (!Overlap(fat[p], Fq)) return;
        const int k = atomicAdd(pairCount, 1);
        const unsigned long long lo = (unsigned long long)(p < q ? p : q), hi = (unsigned long long)(p < q ? q : p);
        if (k < d.pairCap) pairs[k] = (lo << 32) | hi;
    };
    // a list walk visits at most every live proxy once; a longer one would mean broken links
    auto walk = [&](int c, int q, const float4& Fq) {
        int guard = 0;
        for (int p = gridHead[c]; p >= 0; p = gridNext[p]) {
            if (++guard > nLive) { atomicOr(&st->error, kErrInvalid); break; }
            test(p, q, Fq);
        }
    };
    for (int t = tid(); t < m; t += nthreads()) {
        const int q = movedList[t];
        const float4 Fq = fat[q];
        if (size(Fq) > wLarge) {
            const int slot = atomicAdd(&sNLargeQ, 1);
            if (slot < kLargeCap) sLargeQ[slot] = q;
            else for (int j = 0; j < nLive; ++j) test(gridIds[j], q, Fq);
            continue;
        }
        const float lowX = Fq.x - W - 1e-4f * fabsf(Fq.x), lowY = Fq.y - W - 1e-4f * fabsf(Fq.y);
        const int cx0 = max(cellOf(lowX, ox, nx), 0), cx1 = min(cellOf(Fq.z, ox, nx), nx - 1);
        const int cy0 = max(cellOf(lowY, oy, ny), 0), cy1 = min(cellOf(Fq.w, oy, ny), ny - 1);
        for (int cy = cy0; cy <= cy1; ++cy)
            for (int cx = cx0; cx <= cx1; ++cx) walk(cy * nx + cx, q, Fq);
        walk(nCells, q, Fq);
    }
    __syncthreads();
    const int nLarge = min(sNLargeQ, kLargeCap);
    for (int l = 0; l < nLarge; ++l) {
        const int q = sLargeQ[l];
        const float4 Fq = fat[q];
        for (int j = tid(); j < nLive; j += nthreads()) test(gridIds[j], q, Fq);
    }
    __syncthreads();
}

// knownMoved >= 0: movedList already holds that many moved proxies (a continuous-phase event lists
// the proxies its synchronisation moves), so the proxy range is not scanned for them.
__device__ void Wd::findNewContacts(bool inToi, int knownMoved)
{
    __shared__ int sMoved, sPairs, sNew, sKept, sLive, sEventGrid;
    if (tid() == 0) {
        sMoved = 0; sPairs = 0; sNew = 0;
        // a continuous-phase event queries the grid the step kept; any other call builds it anew
        sEventGrid = inToi && st->gridValid ? 1 : 0;
        if (!inToi) st->gridValid = 0;
    }
    __syncthreads();
    const unsigned long long tPairs0 = clock64();
    const int np = d.proxyCap;
    if (knownMoved < 0) {
        for (int p0 = 0; p0 < np; p0 += nthreads()) {
            const int p = p0 + tid();
            const int i = WarpAppend(p < np && moved[p] != 0, &sMoved);
            if (i >= 0) movedList[i] = p;
        }
    }
    __syncthreads();
    const int m = knownMoved < 0 ? sMoved : knownMoved;
    // Query every moved proxy's fat AABB against all proxies (b2BroadPhase.h:188-217); a pair whose
    // both proxies moved is emitted once, from the lower proxy id. Proxy ids are tree node ids, so
    // about half the id range is internal nodes: the live proxies (those with a fixture) are listed
    // first and only they are tested. When they fit, their boxes, ids and moved flags are staged in
    // shared memory (each is read once per moved proxy). The list's order is free: the pairs are
    // sorted below.
    const bool staged = np * (int)(sizeof(float4) + sizeof(int) + 1) <= smemBytes;
    float4* sFat = smemBase;
    int* sId = reinterpret_cast<int*>(smemBase + np);
    unsigned char* sMovedFlag = reinterpret_cast<unsigned char*>(sId + np);
    int* liveList = staged ? sId : liveProxies;
    if (tid() == 0) sLive = 0;
    __syncthreads();
    if (m > 0 && !sEventGrid) {
        for (int p0 = 0; p0 < np; p0 += nthreads()) {
            const int p = p0 + tid();
            const int i = WarpAppend(p < np && pfix[p] >= 0, &sLive);
            if (i < 0) continue;
            liveList[i] = p;
            if (staged) {
                sFat[i] = fat[p];
                sMovedFlag[i] = (unsigned char)(moved[p] != 0);
            }
        }
    }
    __syncthreads();
    const int nLive = sLive;
    const long long total = (long long)m * nLive;
    if (sEventGrid) {
        if (m > 0) gridEventPairs(m, &sPairs);
    } else if (total > kSweepThreshold) {
        __syncthreads();
        gridPairs(m, &sPairs);
    } else
    for (long long idx = tid(); idx < total; idx += nthreads()) {
        const int q = movedList[idx / nLive];
        const int i = (int)(idx % nLive);
        const int p = liveList[i];
        if (p == q) continue;
        if (staged) {
            if (sMovedFlag[i] && p < q) continue;
            if (!Overlap(sFat[i], fat[q])) continue;
        } else {
            if (moved[p] && p < q) continue;
            if (!Overlap(fat[p], fat[q])) continue;
        }
        int k = atomicAdd(&sPairs, 1);
        unsigned long long lo = (unsigned long long)(p < q ? p : q), hi = (unsigned long long)(p < q ? q : p);
        if (k < d.pairCap) pairs[k] = (lo << 32) | hi;
    }
    __syncthreads();
    int n = sPairs;
    if (tid() == 0) st->pairsFound += n;
    if (n > d.pairCap) {
        if (tid() == 0) atomicOr(&st->error, kErrCapacity);
        n = d.pairCap;
    }
    // sort (b2BroadPhase.h:220: std::sort by (proxyIdA, proxyIdB)); in shared memory when it fits
    {
        int P2 = 1;
        while (P2 < n) P2 <<= 1;
        if (n > 1 && P2 * (int)sizeof(unsigned long long) <= smemBytes) {
            unsigned long long* sKeys = reinterpret_cast<unsigned long long*>(smemBase);
            for (int i = tid(); i < n; i += nthreads()) sKeys[i] = pairs[i];
            __syncthreads();
            ctaSortKeys(sKeys, n, P2);
            for (int i = tid(); i < n; i += nthreads()) pairs[i] = sKeys[i];
            __syncthreads();
        } else if (n > 1 && RadixSortFits(n, smemBytes)) {
            // the pair-info scratch is free until contact creation: the radix sort's buffer; its work
            // arrays in the shared memory (free again once the pairs are found)
            ctaRadixSort(pairs, reinterpret_cast<unsigned long long*>(pairInfo), n, reinterpret_cast<int*>(smemBase));
        } else if (n > 1) {
            ctaSortKeys(pairs, n, d.pairCap);
        }
    }
    // b2ContactManager::AddPair checks (Dynamics/b2ContactManager.cpp:179-227), independent per pair.
    for (int k = tid(); k < n; k += nthreads()) {
        int pA = (int)(pairs[k] >> 32), pB = (int)(pairs[k] & 0xffffffffu);
        int fA = pfix[pA], fB = pfix[pB];
        int bA = fixBody(fA), bB = fixBody(fB);
        int keep = 1;
        if (bA == bB) keep = 0;
        if (keep) {
            B2G_WALK(e, bi[bB].w, eNext(e), 2 * d.contactCap + 2) {
                if (edgeOther(e) == bA) {
                    int4 c = ci[e >> 1];
                    if ((c.y == fA && c.z == fB) || (c.y == fB && c.z == fA)) { keep = 0; break; }
                }
            }
        }
        if (keep && !shouldCollide(bB, bA)) keep = 0;
        if (keep && !filterCollide(fA, fB)) keep = 0;
        if (keep && shape[fA].type == kEdge && shape[fB].type == kEdge) keep = 0;
        pairKeep[k] = keep;
    }
    __syncthreads();
    // kept pairs in sorted order, with everything a new contact needs that does not depend on the
    // creation order worked out in parallel: fixtures in factory order, bodies, mixed friction and
    // restitution, and whether the pair wakes its bodies
    int* keptIdx = sContact;
    {
        // indices of the kept pairs, in sorted order (order-preserving compaction over the CTA)
        const int T = nthreads(), t = tid();
        const int chunk = (n + T - 1) / T;
        const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
        int o = 0, u1 = 0, u2 = 0, tot[3];
        for (int k = lo; k < hi; ++k) o += pairKeep[k] != 0;
        ctaExclusiveScan3(o, u1, u2, tot);
        if (t == 0) sKept = tot[0];
        for (int k = lo; k < hi; ++k)
            if (pairKeep[k] && o < d.contactCap) keptIdx[o++] = k;
        __syncthreads();
    }
    // more new contacts than contact slots cannot be created: those beyond the capacity are an overflow
    // here, and the free list runs dry below when fewer slots are free
    const int nKept = min(sKept, d.contactCap);
    if (sKept > d.contactCap && tid() == 0) atomicOr(&st->error, kErrCapacity);
    int4* info = pairInfo;
    for (int r = tid(); r < nKept; r += nthreads()) {
        const int k = keptIdx[r];
        const int pA = (int)(pairs[k] >> 32), pB = (int)(pairs[k] & 0xffffffffu);
        int fa = pfix[pA], fb = pfix[pB];
        if (!primaryOrder(shape[fa].type, shape[fb].type)) { int t = fa; fa = fb; fb = t; }
        const int wake = (fi[fa].w == 0 && fi[fb].w == 0) ? 1 : 0;
        info[r] = make_int4(fa | (wake << 30), fb, fixBody(fa), fixBody(fb));
    }
    __syncthreads();
    const unsigned long long tCreate0 = clock64();
    // Create in sorted pair order; each new contact goes to the front of both bodies' lists
    // (b2ContactManager.cpp:229-293). The list heads of the bodies live in shared memory for the
    // loop when they fit, so only the free-list pop reads global memory on the order-defining path.
    const int nb = d.bodyCount;
    const bool headsStaged = nKept > 0 && nb * (int)sizeof(int) <= smemBytes;
    int* sHead = reinterpret_cast<int*>(smemBase);
    if (headsStaged) {
        for (int b = tid(); b < nb; b += nthreads()) sHead[b] = bi[b].w;
        __syncthreads();
    }
    if (tid() == 0) {
        int created = 0;
        int freeHead = st->freeContact;
        for (int r = 0; r < nKept; ++r) {
            const int4 I = info[r];
            const int fa = I.x & 0x3fffffff, fb = I.y, bA = I.z, bB = I.w;
            const int c = freeHead;
            if (c == kNullIdx) { atomicOr(&st->error, kErrCapacity); break; }
            freeHead = cnext[c];
            const float4 ma = fm[fa], mb = fm[fb];
            ci[c] = make_int4(kCEnabled, fa, fb, 0);
            cp[c] = make_float4(sqrtf(ma.x * mb.x), ma.y > mb.y ? ma.y : mb.y, 0.0f, 1.0f);
            mh[c] = make_int4(0, 0, 0, 0);
            mv[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            mp0[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            mp1[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const int eA = 2 * c, eB = 2 * c + 1;
            const int hA = headsStaged ? sHead[bA] : bi[bA].w;
            if (hA != kNullIdx) *ePrevP(hA) = eA;
            if (headsStaged) sHead[bA] = eA; else bi[bA].w = eA;
            const int hB = headsStaged ? sHead[bB] : bi[bB].w;
            ce[c] = make_int4(kNullIdx, hA, kNullIdx, hB);
            if (hB != kNullIdx) *ePrevP(hB) = eB;
            if (headsStaged) sHead[bB] = eB; else bi[bB].w = eB;
            sContact[created++] = c;
        }
        st->freeContact = freeHead;
        sNew = created;
    }
    __syncthreads();
    const int created = sNew;
    if (headsStaged) {
        for (int b = tid(); b < nb; b += nthreads()) bi[b].w = sHead[b];
    }
    // b2Body::SetAwake(true) of both bodies of every non-sensor pair: idempotent, so in parallel
    for (int r = tid(); r < created; r += nthreads()) {
        const int4 I = info[r];
        if ((I.x >> 30) & 1) {
            setAwake(I.z, true);
            setAwake(I.w, true);
        }
    }
    __syncthreads();
    // order = reverse(new) ++ order: the new contacts go in front of the list's first row; when the
    // rows in front have run out, the list first moves to the end of the world's 2 x contactCap rows
    // (the pair-keep flags are dead now: the copy buffer)
    if (created > 0) {
        const int live = st->contactCount;
        int start = st->orderStart;
        if (start < created) {
            int* tmp = pairKeep;
            for (int i = tid(); i < live; i += nthreads()) tmp[i] = order[i];
            __syncthreads();
            start = 2 * d.contactCap - live;
            for (int i = tid(); i < live; i += nthreads()) orderBase[start + i] = tmp[i];
        }
        start -= created;
        for (int i = tid(); i < created; i += nthreads()) orderBase[start + created - 1 - i] = sContact[i];
        __syncthreads();
        order = orderBase + start;
        if (tid() == 0) {
            st->orderStart = start;
            st->contactCount = live + created;
        }
    }
    for (int i = tid(); i < m; i += nthreads()) moved[movedList[i]] = 0;
    __syncthreads();
    if (tid() == 0) {
        const unsigned long long now = clock64();
        st->cyc[14] += tCreate0 - tPairs0;
        st->cyc[15] += now - tCreate0;
    }
}

// ------------------------------------------------------------------ destroy
// b2ContactManager::Destroy (Dynamics/b2ContactManager.cpp:39-105); wakes are applied by the caller.
__device__ void Wd::destroyContact(int c)
{
    int4 info = ci[c];
    int bA = fixBody(info.y), bB = fixBody(info.z);
    for (int side = 0; side < 2; ++side) {
        int body = side == 0 ? bA : bB;
        int e = 2 * c + side;
        int4 v = ce[c];
        int pe = side == 0 ? v.x : v.z, ne = side == 0 ? v.y : v.w;
        if (pe != kNullIdx) *eNextP(pe) = ne;
        if (ne != kNullIdx) *ePrevP(ne) = pe;
        if (bi[body].w == e) bi[body].w = ne;
    }
    ci[c].x = 0;
    cnext[c] = st->freeContact;
    st->freeContact = c;
}

// ------------------------------------------------------------------ Collide
// b2ContactManager::Collide (Dynamics/b2ContactManager.cpp:107-172). The reference walks the contact
// list once; a contact is processed only if one of its bodies is awake and non-static at that point,
// and processing can wake bodies for contacts later in the list. Evaluation results do not depend on
// the order, so all contacts are evaluated in parallel and the wake chain is resolved as a fixpoint:
// body b is awake for list position k iff it was awake at the start or a processed contact at a
// position < k woke it.
__device__ void Wd::collide()
{
    __shared__ int sChanged;
    const int n = st->contactCount;
    // manifolds NarrowphaseKernel evaluated for this step (cleared below once committed)
    const bool staged = st->staged != 0;
    // two shape slots per thread in the dynamic shared memory (free during this phase) when it fits
    Shape* shapeSlots = (int)(2 * sizeof(Shape)) * nthreads() <= smemBytes ? reinterpret_cast<Shape*>(smemBase) : nullptr;
    for (int b = tid(); b < d.bodyCount; b += nthreads()) sWake[b] = awake(b) ? -1 : INT_MAX;
    const bool rec = evLog != nullptr;
    for (int k = tid(); k < n; k += nthreads()) { sStatus[k] = 0; evType[k] = 0; }
    __syncthreads();
    for (int round = 0; round <= n + 1; ++round) {
        if (tid() == 0) sChanged = 0;
        __syncthreads();
        for (int k = tid(); k < n; k += nthreads()) {
            if (sStatus[k] != 0) continue;
            int c = order[k];
            int4 info = ci[c];
            int bA = fixBody(info.y), bB = fixBody(info.z);
            bool sensor = fi[info.y].w != 0 || fi[info.z].w != 0;
            if (info.x & kCFilter) {
                bool keep = shouldCollide(bB, bA) && filterCollide(info.y, info.z);
                if (!keep) {
                    sStatus[k] = 2;
                    if (rec && (info.x & kCTouching)) evType[k] = 2;
                    if (mh[c].y > 0 && !sensor) {
                        if (atomicMin(&sWake[bA], k) > k) sChanged = 1;
                        if (atomicMin(&sWake[bB], k) > k) sChanged = 1;
                    }
                    continue;
                }
                ci[c].x = info.x & ~kCFilter;
            }
            bool activeA = type(bA) != kStatic && sWake[bA] < k;
            bool activeB = type(bB) != kStatic && sWake[bB] < k;
            if (!activeA && !activeB) continue;
            if (!Overlap(fat[fi[info.y].z], fat[fi[info.z].z])) {
                sStatus[k] = 2;
                if (rec && (info.x & kCTouching)) evType[k] = 2;
                if (mh[c].y > 0 && !sensor) {
                    if (atomicMin(&sWake[bA], k) > k) sChanged = 1;
                    if (atomicMin(&sWake[bB], k) > k) sChanged = 1;
                }
                continue;
            }
            sStatus[k] = 1;
            const bool updated = update(c, shapeSlots ? shapeSlots + 2 * tid() : nullptr, staged);
            if (rec) evType[k] = updateEventBits((info.x & kCTouching) != 0, (ci[c].x & kCTouching) != 0, sensor);
            if (updated) {
                if (atomicMin(&sWake[bA], k) > k) sChanged = 1;
                if (atomicMin(&sWake[bB], k) > k) sChanged = 1;
            }
        }
        __syncthreads();
        if (sChanged == 0) break;
    }
    for (int b = tid(); b < d.bodyCount; b += nthreads()) {
        int wk = sWake[b];
        if (wk != -1 && wk != INT_MAX) setAwake(b, true);
    }
    __syncthreads();
    // Listener calls of the collide phase in list order (b2ContactManager::Collide visits the list in
    // order; each contact's Update or Destroy makes its calls), appended to the event log.
    if (rec) {
        const int T = nthreads(), t = tid();
        const int chunk = (n + T - 1) / T;
        const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
        int slot = 0, u1 = 0, u2 = 0, tot[3];
        for (int k = lo; k < hi; ++k) slot += __popc(evType[k] & 7);
        const int base = st->eventCount;
        ctaExclusiveScan3(slot, u1, u2, tot);
        slot += base;
        for (int k = lo; k < hi; ++k) {
            const int bits = evType[k] & 7;
            if (!bits) continue;
            const int4 info = ci[order[k]];
            for (int b = 0; b < 3; ++b)
                if (bits & (1 << b)) putEvent(slot++, b, info.y, info.z);
        }
        __syncthreads();
        if (t == 0) st->eventCount = base + tot[0];
        __syncthreads();
    }
    // Survivors keep their relative order; destroyed contacts are unlinked in list order.
    int* kept = sContact;
    int* gone = pairKeep;
    const int nKept = ctaCompact(order, n, kept, [&](int k) { return sStatus[k] != 2; });
    const int nGone = ctaCompact(order, n, gone, [&](int k) { return sStatus[k] == 2; });
    if (tid() == 0) {
        for (int i = 0; i < nGone; ++i) destroyContact(gone[i]);
        st->contactCount = nKept;
        st->staged = 0;
    }
    for (int k = tid(); k < nKept; k += nthreads()) order[k] = kept[k];
    __syncthreads();
}

#include "b2g_solver.cuh"

// ------------------------------------------------------------------ Solve
// b2World::Solve (Dynamics/b2World.cpp:388-577). The island DFS runs on one thread (it fixes the
// contact order inside every island); islands are then solved in parallel, one per thread, because
// they share no dynamic body.
// The island DFS of b2World::Solve (Dynamics/b2World.cpp:422-510) from a table: a parallel pre-pass
// flattens the edge list of every non-static body into a table of its eligible contacts (enabled,
// touching, no sensor) in list order, and copies the body-list links and body flags; thread 0 then
// runs the DFS on that table. Contacts, joints and bodies are visited in exactly the order of the
// global DFS, so islands, rows and contact order (and colours) are the same; island flags, wakes and
// contact island flags are written back in parallel afterwards (they are idempotent and nothing in
// the DFS reads them back from global memory).
// Two table layouts: IslPacked (16-bit body and 15-bit contact indices, four bytes per entry) in the
// CTA's shared memory, and IslWide (32-bit indices) in the world's global table region, for worlds
// whose packed table does not fit or whose indices do not pack.
// Returns false (nothing written outside the table region) when the world does not fit the layout.
struct IslPacked {
    using Idx = unsigned short;
    using Entry = unsigned;
    using Pair = unsigned;
    static constexpr int kMaxBodies = 65536, kMaxContacts = 32768;
    __device__ static Entry entry(int c, int side, int other) { return ((unsigned)c << 17) | ((unsigned)side << 16) | (unsigned)other; }
    __device__ static int contact(Entry u) { return (int)(u >> 17); }
    __device__ static int side(Entry u) { return (int)((u >> 16) & 1u); }
    __device__ static int other(Entry u) { return (int)(u & 0xffffu); }
    __device__ static Pair pair(int a, int b) { return (unsigned)a | ((unsigned)b << 16); }
    __device__ static int pairA(Pair p) { return (int)(p & 0xffffu); }
    __device__ static int pairB(Pair p) { return (int)(p >> 16); }
    // a contact's dynamic bodies for the colouring (kNone: static or kinematic)
    static constexpr int kNone = 0xffff;
    __device__ static Entry cinfo(int a, int b) { return (unsigned)a | ((unsigned)b << 16); }
    __device__ static int cinfoA(Entry u) { return (int)(u & 0xffffu); }
    __device__ static int cinfoB(Entry u) { return (int)(u >> 16); }
};
struct IslWide {
    using Idx = int;
    using Entry = int2;
    using Pair = int2;
    static constexpr int kMaxBodies = 1 << 30, kMaxContacts = 1 << 29;
    __device__ static Entry entry(int c, int side, int other) { return make_int2((c << 1) | side, other); }
    __device__ static int contact(Entry u) { return u.x >> 1; }
    __device__ static int side(Entry u) { return u.x & 1; }
    __device__ static int other(Entry u) { return u.y; }
    __device__ static Pair pair(int a, int b) { return make_int2(a, b); }
    __device__ static int pairA(Pair p) { return p.x; }
    __device__ static int pairB(Pair p) { return p.y; }
    static constexpr int kNone = -1;
    __device__ static Entry cinfo(int a, int b) { return make_int2(a, b); }
    __device__ static int cinfoA(Entry u) { return u.x; }
    __device__ static int cinfoB(Entry u) { return u.y; }
};

template <class L>
__device__ bool Wd::buildIslandsTable(unsigned char* base, int capacity, bool coloured, int* colourCount, int& nIslOut,
                                      int& nRowsOut, int& nConsOut, int& moversOut)
{
    using Idx = typename L::Idx;
    using Entry = typename L::Entry;
    using Pair = typename L::Pair;
    __shared__ int sE, sOk, sIsl, sRowsS, sConsS, sMovers;
    enum : unsigned char { fIsl = 1, fStatic = 2, fAwake = 4, fActive = 8, fDynamic = 16, fJoints = 32 };
    const int nb = d.bodyCount, C = d.contactCap;
    if (!base || nb >= L::kMaxBodies || C >= L::kMaxContacts || nb == 0) return false;
    // layout (bytes): masks 8nb | off 4(nb+1) | next 4nb | stack 4nb | cbits 4ceil(C/32) | local |
    // statics | bflag nb | entries E | island contact pairs E (a contact with a static body has one entry)
    auto up = [](long long x) { return (x + 7) & ~7ll; };
    const long long oMask = 0;
    const long long oOff = oMask + (coloured ? 8ll * nb : 0);
    const long long oNext = oOff + 4ll * (nb + 1);
    const long long oStack = oNext + 4ll * nb;
    const long long oBits = oStack + 4ll * nb;
    const long long oLocal = up(oBits + 4ll * ((C + 31) / 32));
    const long long oStatics = up(oLocal + (long long)sizeof(Idx) * nb);
    const long long oFlag = up(oStatics + (long long)sizeof(Idx) * nb);
    const long long oEntries = up(oFlag + nb);
    if (oEntries > capacity) return false;
    unsigned long long* mask = reinterpret_cast<unsigned long long*>(base + oMask);
    int* off = reinterpret_cast<int*>(base + oOff);
    int* next = reinterpret_cast<int*>(base + oNext);
    int* stack = reinterpret_cast<int*>(base + oStack);
    unsigned* cbits = reinterpret_cast<unsigned*>(base + oBits);
    Idx* local = reinterpret_cast<Idx*>(base + oLocal);
    Idx* statics = reinterpret_cast<Idx*>(base + oStatics);
    unsigned char* bflag = base + oFlag;
    Entry* entries = reinterpret_cast<Entry*>(base + oEntries);
    auto eligible = [&](int e, int& other) {
        const int4 info = ci[e >> 1];
        other = (e & 1) == 0 ? fixBody(info.z) : fixBody(info.y);
        return (info.x & kCEnabled) != 0 && (info.x & kCTouching) != 0 && fi[info.y].w == 0 && fi[info.z].w == 0;
    };
    // pre-pass 1: flags, links, eligible-edge counts
    for (int b = tid(); b < nb; b += nthreads()) {
        const int4 B = bi[b];
        unsigned char f = 0;
        if (B.x == kStatic) f |= fStatic;
        if (B.x == kDynamic) f |= fDynamic;
        if (B.y & kBAwake) f |= fAwake;
        if (B.y & kBActive) f |= fActive;
        if (bj[b].x != kNullIdx) f |= fJoints;
        bflag[b] = f;
        next[b] = bj[b].y;
        int cnt = 0;
        if (B.x != kStatic) {
            B2G_WALK(e, B.w, eNext(e), 2 * C + 2) {
                int other;
                if (eligible(e, other)) ++cnt;
            }
        }
        off[b + 1] = cnt;
    }
    for (int k = tid(); k < (C + 31) / 32; k += nthreads()) cbits[k] = 0u;
    __syncthreads();
    if (tid() == 0) {
        off[0] = 0;
        for (int b = 0; b < nb; ++b) off[b + 1] += off[b];
        const long long E = off[nb];
        sE = (int)E;
        // the table, then one pair slot per possible island contact
        sOk = oEntries + (long long)(sizeof(Entry) + sizeof(Pair)) * E + 8 <= capacity ? 1 : 0;
    }
    __syncthreads();
    if (!sOk) return false;
    const int E = sE;
    Pair* icPairs = reinterpret_cast<Pair*>(entries + E);
    // pre-pass 2: the table, {contact, side, other body} in list order
    for (int b = tid(); b < nb; b += nthreads()) {
        if (bflag[b] & fStatic) continue;
        int k = off[b];
        B2G_WALK(e, bi[b].w, eNext(e), 2 * C + 2) {
            int other;
            if (eligible(e, other)) entries[k++] = L::entry(e >> 1, e & 1, other);
        }
    }
    __syncthreads();
    if (tid() == 0) {
        int nIsl = 0, bCur = 0, cCur = 0, jCur = 0, movers = 0, guard = 0;
        for (int seed = st->bodyList; seed != kNullIdx; seed = next[seed]) {
            if (++guard > nb) { atomicOr(&st->error, kErrInvalid); break; }
            const unsigned char fl = bflag[seed];
            if (fl & fIsl) continue;
            if ((fl & fAwake) == 0 || (fl & fActive) == 0) continue;
            if (fl & fStatic) continue;
            const int bStart = bCur, cStart = cCur, jStart = jCur;
            int stackCount = 0, nStatics = 0;
            stack[stackCount++] = seed;
            bflag[seed] = fl | fIsl;
            while (stackCount > 0) {
                const int b = stack[--stackCount];
                if (bCur >= d.rowCap) { atomicOr(&st->error, kErrCapacity); stackCount = 0; break; }
                const int loc = bCur - bStart;
                local[b] = (Idx)loc;
                bj[b].z = loc;
                if (coloured) mask[loc] = 0ull;
                sBody[bCur++] = b;
                const unsigned char fb = bflag[b];
                if (fb & fStatic) { statics[nStatics++] = (Idx)b; continue; }
                ++movers;
                for (int k = off[b], ke = off[b + 1]; k < ke; ++k) {
                    const Entry u = entries[k];
                    const int c = L::contact(u), other = L::other(u);
                    const unsigned bit = 1u << (c & 31);
                    if (cbits[c >> 5] & bit) continue;
                    cbits[c >> 5] |= bit;
                    icPairs[cCur - cStart] = L::side(u) ? L::pair(other, b) : L::pair(b, other);
                    sContact[cCur++] = c;
                    if (bflag[other] & fIsl) continue;
                    stack[stackCount++] = other;
                    bflag[other] |= fIsl;
                }
                if (fb & fJoints) {
                    B2G_WALK(e, bj[b].x, jNext(e), 2 * d.jointCount + 2) {
                        Joint& J = jt[e >> 1];
                        if (J.islandFlag) continue;
                        const int other = jOther(e);
                        if ((bflag[other] & fActive) == 0) continue;
                        sJoint[jCur++] = e >> 1;
                        J.islandFlag = 1;
                        if (bflag[other] & fIsl) continue;
                        stack[stackCount++] = other;
                        bflag[other] |= fIsl;
                    }
                }
            }
            islands[nIsl] = make_int4(bStart, bCur - bStart, cStart, cCur - cStart);
            islandJ[nIsl] = make_int2(jStart, jCur - jStart);
            ++nIsl;
            for (int i = cStart; i < cCur; ++i) {
                const Pair pr = icPairs[i - cStart];
                const int bA = L::pairA(pr), bB = L::pairB(pr);
                const int lA = local[bA], lB = local[bB];
                vc[i].idx = make_int4(bStart + lA, bStart + lB, 0, 0);
                if (coloured) {
                    const bool dA = (bflag[bA] & fDynamic) != 0, dB = (bflag[bB] & fDynamic) != 0;
                    const unsigned long long used = (dA ? mask[lA] : 0ull) | (dB ? mask[lB] : 0ull);
                    const unsigned long long freeBits = ~used & ((1ull << kSerialColour) - 1ull);
                    const int col = freeBits ? __ffsll((long long)freeBits) - 1 : kSerialColour;
                    if (col != kSerialColour) {
                        if (dA) mask[lA] |= 1ull << col;
                        if (dB) mask[lB] |= 1ull << col;
                    }
                    cColour[i] = col;
                    ++colourCount[col];
                }
            }
            for (int i = jStart; i < jCur; ++i) {
                Joint& J = jt[sJoint[i]];
                J.indexA = bStart + local[J.bodyA];
                J.indexB = bStart + local[J.bodyB];
                if (J.type == kJointGear) {
                    // the coupled joints, and with them bodies C and D, are in the same island
                    J.indexC = bStart + local[J.bodyC];
                    J.indexD = bStart + local[J.bodyD];
                }
            }
            for (int i = 0; i < nStatics; ++i) bflag[statics[i]] &= (unsigned char)~fIsl;
        }
        sIsl = nIsl;
        sRowsS = bCur;
        sConsS = cCur;
        sMovers = movers;
    }
    __syncthreads();
    const int nRows = sRowsS, nCons = sConsS;
    // write-back: body island flags, then wakes (b2Body::SetAwake(true) of every island body), then
    // the island flag of every island contact
    for (int b = tid(); b < nb; b += nthreads()) {
        const int y = bi[b].y;
        bi[b].y = (bflag[b] & fIsl) ? (y | kBIsland) : (y & ~kBIsland);
    }
    __syncthreads();
    for (int r = tid(); r < nRows; r += nthreads()) setAwake(sBody[r], true);
    for (int i = tid(); i < nCons; i += nthreads()) ci[sContact[i]].x |= kCIsland;
    __syncthreads();
    nIslOut = sIsl;
    nRowsOut = nRows;
    nConsOut = nCons;
    moversOut = sMovers;
    return true;
}

// Island build of the graph-coloured solver, spread over the CTA. That solver does not depend on the
// order in which b2World::Solve's depth-first search (Dynamics/b2World.cpp:410-497) visits bodies and
// contacts, only on which bodies, contacts and joints form each island, so the islands are built as
// connected components instead of by the search:
//   * the same eligible edges as the search (touching, enabled, non-sensor contacts, taken flat from
//     the world's contact list; joints whose bodies are active) join non-static bodies by union-find
//     (a root is linked under the smaller root, so each component's root is its smallest body index
//     whatever the schedule);
//   * a component is an island when it holds an awake, active, non-static body (a search seed); the
//     islands are numbered by root;
//   * one 64-bit key per island member, (island, kind, index) with kind 0 non-static body, 1 static
//     body (one row per island that reaches it, as the search gives it), 2 contact, 3 joint, sorted
//     once: each island's rows, contacts and joints in index order;
//   * contacts are coloured by rounds of a parallel greedy colouring (Jones-Plassmann): an uncoloured
//     contact whose hashed key is the smallest among the uncoloured contacts at each of its dynamic
//     bodies takes the lowest colour neither body holds yet. Every result is a function of the world
//     state alone, not of thread timing or count.
// Returns false (nothing written outside the scratch) when the scratch does not fit; the caller then
// takes the search.

// The colouring's key of island contact i in round gr: rounds count down in the top 16 bits (a later
// round's key is smaller than any earlier one), then a 16-bit hash of i (the priority order), then i
// (unique keys).
__device__ inline unsigned long long ColourKey(int i, int gr)
{
    unsigned h = (unsigned)i * 0x9E3779B1u;
    h ^= h >> 15;
    h *= 0x85EBCA77u;
    h ^= h >> 13;
    return ((unsigned long long)(0xffffu - (unsigned)gr) << 48) | ((unsigned long long)(h & 0xffffu) << 32) |
           (unsigned)i;
}

template <class L>
__device__ bool Wd::buildIslandsParallel(unsigned char* base, int capacity, int* radixWork, int* colourCount,
                                         int& nIslOut, int& nRowsOut, int& nConsOut, int& moversOut)
{
    using Entry = typename L::Entry;
    __shared__ int sN, sMovers, sFlags[4];
    enum : unsigned char { fStatic = 2, fAwake = 4, fActive = 8, fDynamic = 16 };
    const int nb = d.bodyCount, C = d.contactCap, NJ = d.jointCount;
    const int T = nthreads(), t = tid();
    if (!base || nb == 0 || nb >= L::kMaxBodies || C >= L::kMaxContacts || T > kMaxCta) return false;
    const unsigned long long tBuild0 = clock64();
    const int nc = st->contactCount;
    auto up = [](long long x) { return (x + 15) & ~15ll; };
    // layout (bytes): flags nb | parent 4nb | island 4nb | row 4nb | static rows 4nb | colours used 8nb
    // | owner 8nb | colour nc | dynamic bodies of each island contact nc x Entry (the colour masks and
    // owners, contiguous, first hold the island extents: 12 bytes per island)
    const long long oFlag = 0;
    const long long oParent = up(oFlag + nb);
    const long long oIsl = up(oParent + 4ll * nb);
    const long long oRow = up(oIsl + 4ll * nb);
    const long long oSStart = up(oRow + 4ll * nb);
    const long long oUsed = up(oSStart + 4ll * nb);
    const long long oOwner = up(oUsed + 8ll * nb);
    const long long oCol = up(oOwner + 8ll * nb);
    const long long oCinf = up(oCol + nc);
    if (oCinf + (long long)sizeof(Entry) * nc > capacity) return false;
    unsigned char* bflag = base + oFlag;
    int* parent = reinterpret_cast<int*>(base + oParent);
    int* islOf = reinterpret_cast<int*>(base + oIsl);
    int* rowOf = reinterpret_cast<int*>(base + oRow);
    int* sStart = reinterpret_cast<int*>(base + oSStart);
    unsigned long long* used = reinterpret_cast<unsigned long long*>(base + oUsed);
    unsigned long long* owner = reinterpret_cast<unsigned long long*>(base + oOwner);
    signed char* ccol = reinterpret_cast<signed char*>(base + oCol);
    Entry* cinf = reinterpret_cast<Entry*>(base + oCinf);
    // a live contact joins its bodies when b2World::Solve's search would follow it
    auto eligible = [&](const int4& info) {
        return (info.x & kCEnabled) != 0 && (info.x & kCTouching) != 0 && fi[info.y].w == 0 && fi[info.z].w == 0;
    };
    for (int b = t; b < nb; b += T) {
        const int4 B = bi[b];
        unsigned char f = 0;
        if (B.x == kStatic) f |= fStatic;
        if (B.x == kDynamic) f |= fDynamic;
        if (B.y & kBAwake) f |= fAwake;
        if (B.y & kBActive) f |= fActive;
        bflag[b] = f;
        parent[b] = b;
    }
    if (t == 0) sN = 0;
    __syncthreads();
    // union-find over the edges between non-static bodies. find halves the path it walks (a node
    // that is not a root takes its grandparent, still an ancestor; roots change only by the linking
    // compare-and-swap); every loop is bounded by the body count.
    volatile int* vp = parent;
    auto find = [&](int x) {
        for (int g = 0; g <= nb; ++g) {
            const int p = vp[x];
            if (p == x) break;
            const int gp = vp[p];
            if (gp != p) vp[x] = gp;
            x = gp;
        }
        return x;
    };
    auto unite = [&](int a, int b) {
        for (int g = 0; g <= 2 * nb; ++g) {
            a = find(a);
            b = find(b);
            if (a == b) return;
            if (a > b) { const int x = a; a = b; b = x; }
            if (atomicCAS(&parent[b], b, a) == b) return;
        }
        atomicOr(&st->error, kErrInvalid);
    };
    for (int k = t; k < nc; k += T) {
        const int4 info = ci[order[k]];
        if (!eligible(info)) continue;
        const int bA = fixBody(info.y), bB = fixBody(info.z);
        if (!(bflag[bA] & fStatic) && !(bflag[bB] & fStatic)) unite(bA, bB);
    }
    for (int j = t; j < NJ; j += T) {
        const int A = jt[j].bodyA, B = jt[j].bodyB;
        if (A < 0 || B < 0) continue;  // a destroyed joint's slot
        const unsigned char fa = bflag[A], fb = bflag[B];
        if (!(fa & fStatic) && !(fb & fStatic) && (fa & fActive) && (fb & fActive)) unite(A, B);
    }
    __syncthreads();
    // roots: the trees no longer change, so a read-only walk (no halving) into a separate array,
    // then copied once every walk is done
    for (int b = t; b < nb; b += T) {
        int x = b;
        if (!(bflag[b] & fStatic))
            for (int g = 0; g <= nb && parent[x] != x; ++g) x = parent[x];
        sStart[b] = x;
    }
    __syncthreads();
    for (int b = t; b < nb; b += T) {
        parent[b] = sStart[b];
        islOf[b] = 0;
    }
    __syncthreads();
    // a component is an island when it holds a seed: an awake, active, non-static body
    for (int b = t; b < nb; b += T) {
        const unsigned char f = bflag[b];
        if (!(f & fStatic) && (f & fAwake) && (f & fActive)) islOf[parent[b]] = 1;
    }
    __syncthreads();
    // islands numbered by root, in root order (chunked scan over the bodies)
    int nIsl = 0;
    {
        const int chunk = (nb + T - 1) / T;
        const int lo = min(nb, t * chunk), hi = min(nb, lo + chunk);
        int o = 0, u1 = 0, u2 = 0, tot[3];
        for (int b = lo; b < hi; ++b) o += (!(bflag[b] & fStatic) && parent[b] == b && islOf[b] == 1) ? 1 : 0;
        ctaExclusiveScan3(o, u1, u2, tot);
        nIsl = tot[0];
        for (int b = lo; b < hi; ++b) {
            if (bflag[b] & fStatic) continue;
            if (parent[b] == b) islOf[b] = islOf[b] == 1 ? o++ : -1;
        }
    }
    __syncthreads();
    for (int b = t; b < nb; b += T) {
        if (bflag[b] & fStatic) { islOf[b] = -1; continue; }
        if (parent[b] != b) islOf[b] = islOf[parent[b]];
    }
    __syncthreads();
    // keys (island << 34 | kind << 32 | index) in the pair-key scratch, which the solve does not use;
    // more keys than its capacity returns false
    unsigned long long* keys = pairs;
    unsigned long long* tmp = reinterpret_cast<unsigned long long*>(pairInfo);
    const int keyCap = d.pairCap;
    auto push = [&](int isl, int kind, int index) {
        const int p = atomicAdd(&sN, 1);
        if (p < keyCap) keys[p] = ((unsigned long long)isl << 34) | ((unsigned long long)kind << 32) | (unsigned)index;
    };
    const unsigned long long tKeys0 = clock64();
    for (int b = t; b < nb; b += T)
        if (islOf[b] >= 0) push(islOf[b], 0, b);
    for (int k = t; k < nc; k += T) {
        const int c = order[k];
        const int4 info = ci[c];
        if (!eligible(info)) continue;
        const int bA = fixBody(info.y), bB = fixBody(info.z);
        const bool sA = (bflag[bA] & fStatic) != 0, sB = (bflag[bB] & fStatic) != 0;
        const int isl = !sA ? islOf[bA] : islOf[bB];
        if (isl < 0) continue;
        push(isl, 2, c);
        if (sA) push(isl, 1, bA);
        if (sB) push(isl, 1, bB);
    }
    for (int j = t; j < NJ; j += T) {
        const int A = jt[j].bodyA, B = jt[j].bodyB;
        if (A < 0 || B < 0) continue;  // a destroyed joint's slot
        const unsigned char fa = bflag[A], fb = bflag[B];
        if (!(fa & fActive) || !(fb & fActive)) continue;
        const int isl = !(fa & fStatic) ? islOf[A] : (!(fb & fStatic) ? islOf[B] : -1);
        if (isl < 0) continue;
        push(isl, 3, j);
        if (fa & fStatic) push(isl, 1, A);
        if (fb & fStatic) push(isl, 1, B);
    }
    __syncthreads();
    const int n = sN;
    if (n > keyCap) return false;
    if (radixWork && RadixSortFits(n, RadixWorkInts() * (int)sizeof(int)))
        ctaRadixSort(keys, tmp, n, radixWork);
    else
        ctaSortKeys(keys, n, keyCap);
    __syncthreads();
    const unsigned long long tSort1 = clock64();
    auto kIsl = [&](unsigned long long k) { return (int)(k >> 34); };
    auto kKind = [&](unsigned long long k) { return (int)((k >> 32) & 3ull); };
    auto kIdx = [&](unsigned long long k) { return (int)(k & 0xffffffffull); };
    for (int i = t; i < nIsl; i += T) sStart[i] = -1;
    __syncthreads();
    // rows (non-static bodies, then each distinct static body), contacts and joints in key order:
    // one chunked scan with three counters
    int nRows = 0, nCons = 0, nJ = 0;
    {
        const int chunk = (n + T - 1) / T;
        const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
        int cr = 0, cc = 0, cj = 0;
        for (int k = lo; k < hi; ++k) {
            const unsigned long long key = keys[k];
            const int kind = kKind(key);
            if (kind == 0 || (kind == 1 && (k == 0 || keys[k - 1] != key))) ++cr;
            else if (kind == 2) ++cc;
            else if (kind == 3) ++cj;
        }
        if (t == 0) sMovers = 0;
        int tot[3];
        ctaExclusiveScan3(cr, cc, cj, tot);
        nRows = tot[0];
        nCons = tot[1];
        nJ = tot[2];
        if (nRows > d.rowCap || nCons > nc) return false;
        int r = cr, c = cc, jj = cj;
        int movers = 0;
        for (int k = lo; k < hi; ++k) {
            const unsigned long long key = keys[k];
            const int kind = kKind(key), idx = kIdx(key), isl = kIsl(key);
            const bool first = k == 0 || kIsl(keys[k - 1]) != isl;
            if (first) {
                islands[isl] = make_int4(r, 0, c, 0);
                islandJ[isl] = make_int2(jj, 0);
            }
            if (kind == 0) {
                rowOf[idx] = r;
                sBody[r++] = idx;
                ++movers;
            } else if (kind == 1) {
                if (k > 0 && keys[k - 1] == key) continue;
                if (k == 0 || kKind(keys[k - 1]) != 1 || kIsl(keys[k - 1]) != isl) sStart[isl] = r;
                sBody[r++] = idx;
            } else if (kind == 2) {
                sContact[c++] = idx;
            } else {
                sJoint[jj++] = idx;
            }
        }
        atomicAdd(&sMovers, movers);
    }
    __syncthreads();
    // island extents from the next island's starts, read in one pass and written in the next (the
    // colour masks and owners, not yet in use, hold three counts per island in between); an island
    // without static rows has its static range empty at the end of its rows
    int* extent = reinterpret_cast<int*>(used);
    for (int i = t; i < nIsl; i += T) {
        const int4 I = islands[i];
        const int2 J = islandJ[i];
        extent[3 * i] = (i + 1 < nIsl ? islands[i + 1].x : nRows) - I.x;
        extent[3 * i + 1] = (i + 1 < nIsl ? islands[i + 1].z : nCons) - I.z;
        extent[3 * i + 2] = (i + 1 < nIsl ? islandJ[i + 1].x : nJ) - J.x;
    }
    __syncthreads();
    for (int i = t; i < nIsl; i += T) {
        const int4 I = islands[i];
        islands[i] = make_int4(I.x, extent[3 * i], I.z, extent[3 * i + 1]);
        islandJ[i] = make_int2(islandJ[i].x, extent[3 * i + 2]);
        if (sStart[i] < 0) sStart[i] = I.x + extent[3 * i];
    }
    __syncthreads();
    // row of body b in island isl: its own row, or a binary search over the island's static rows
    auto rowIn = [&](int isl, int b) {
        if (!(bflag[b] & fStatic)) return rowOf[b];
        const int end = islands[isl].x + islands[isl].y;
        int lo = sStart[isl], hi = end;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sBody[mid] < b) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= end || sBody[lo] != b) {
            // every static body an island reaches has a row in it; report and stay in bounds
            atomicOr(&st->error, kErrInvalid);
            return islands[isl].x;
        }
        return lo;
    };
    for (int i = t; i < nCons; i += T) {
        const int4 info = ci[sContact[i]];
        const int bA = fixBody(info.y), bB = fixBody(info.z);
        const int isl = !(bflag[bA] & fStatic) ? islOf[bA] : islOf[bB];
        vc[i].idx = make_int4(rowIn(isl, bA), rowIn(isl, bB), 0, 0);
        ccol[i] = -1;
        cinf[i] = L::cinfo((bflag[bA] & fDynamic) ? bA : L::kNone, (bflag[bB] & fDynamic) ? bB : L::kNone);
        ci[sContact[i]].x = info.x | kCIsland;
    }
    for (int q = t; q < nJ; q += T) {
        Joint& J = jt[sJoint[q]];
        const int isl = !(bflag[J.bodyA] & fStatic) ? islOf[J.bodyA] : islOf[J.bodyB];
        J.islandFlag = 1;
        J.indexA = rowIn(isl, J.bodyA);
        J.indexB = rowIn(isl, J.bodyB);
        if (J.type == kJointGear) {
            J.indexC = rowIn(isl, J.bodyC);
            J.indexD = rowIn(isl, J.bodyD);
        }
    }
    for (int b = t; b < nb; b += T) {
        const int y = bi[b].y;
        const bool inIsland = islOf[b] >= 0;
        bi[b].y = inIsland ? (y | kBIsland) : (y & ~kBIsland);
        if (inIsland) bj[b].z = rowOf[b] - islands[islOf[b]].x;
        used[b] = 0ull;
        owner[b] = ~0ull;
    }
    if (t == 0) { sFlags[0] = sFlags[1] = sFlags[2] = sFlags[3] = 0; }
    __syncthreads();
    for (int r = t; r < nRows; r += T) setAwake(sBody[r], true);
    // colouring in shared memory (Jones-Plassmann): rounds of two passes. Pass A: every uncoloured
    // contact lowers its dynamic bodies' owner keys to its own; pass B: a contact that owns all its
    // dynamic bodies (its key is the smallest among the uncoloured contacts at each) takes the lowest
    // colour that none of its bodies holds yet and marks it on them (no other contact at those bodies
    // wins the round). Keys carry the round in their top bits (later rounds smaller), so owners need
    // no reset; the priority order of the contacts is the same in every round, so each round colours
    // at least the smallest key left. The colouring ends when no contact is uncoloured.
    for (int gr = 0; gr < 4096; ++gr) {
        const int par = gr & 1;
        int unc = 0;
        for (int i = t; i < nCons; i += T) {
            if (ccol[i] >= 0) continue;
            unc = 1;
            const Entry u = cinf[i];
            const int a = L::cinfoA(u), b = L::cinfoB(u);
            const unsigned long long key = ColourKey(i, gr);
            if (a != L::kNone) atomicMin(&owner[a], key);
            if (b != L::kNone) atomicMin(&owner[b], key);
        }
        if (unc) sFlags[par] = 1;
        __syncthreads();
        if (sFlags[par] == 0) break;
        // the other parity's flag was last read before the previous barrier
        if (t == 0) sFlags[par ^ 1] = 0;
        for (int i = t; i < nCons; i += T) {
            if (ccol[i] >= 0) continue;
            const Entry u = cinf[i];
            const int a = L::cinfoA(u), b = L::cinfoB(u);
            const unsigned long long key = ColourKey(i, gr);
            if ((a == L::kNone || owner[a] == key) && (b == L::kNone || owner[b] == key)) {
                const unsigned long long busy = (a != L::kNone ? used[a] : 0ull) | (b != L::kNone ? used[b] : 0ull);
                const unsigned long long freeBits = ~busy & ((1ull << kSerialColour) - 1ull);
                const int col = freeBits ? __ffsll((long long)freeBits) - 1 : kSerialColour;
                ccol[i] = (signed char)col;
                if (col != kSerialColour) {
                    if (a != L::kNone) used[a] |= 1ull << col;
                    if (b != L::kNone) used[b] |= 1ull << col;
                }
            }
        }
        __syncthreads();
    }
    __syncthreads();
    // contacts left over take the serial colour (solved by one thread in island order)
    for (int i = t; i < nCons; i += T) {
        const int c = ccol[i] >= 0 ? ccol[i] : kSerialColour;
        cColour[i] = c;
        atomicAdd(&colourCount[c], 1);
    }
    __syncthreads();
    if (t == 0) {
        st->cyc[22] = tKeys0 - tBuild0;
        st->cyc[23] = tSort1 - tKeys0;
    }
    nIslOut = nIsl;
    nRowsOut = nRows;
    nConsOut = nCons;
    moversOut = sMovers;
    return true;
}

__device__ void Wd::solve(const StepParams& P, float4* smem, int smemRows, int smemContacts)
{
    __shared__ int sIslands, sRows, sCons;
    __shared__ int sColourStart[kColours + 1], sColourCursor[kColours];
    const unsigned long long tSolve0 = clock64();
    const int nb = d.bodyCount, nc = st->contactCount;
    const bool coloured = P.solver == kSolverColoured;
    for (int b = tid(); b < nb; b += nthreads()) bi[b].y &= ~kBIsland;
    for (int k = tid(); k < nc; k += nthreads()) ci[order[k]].x &= ~kCIsland;
    for (int j = tid(); j < d.jointCount; j += nthreads()) jt[j].islandFlag = 0;
    for (int k = tid(); k <= kColours; k += nthreads()) sColourStart[k] = 0;
    __syncthreads();
    // Colour masks of the island body rows while the DFS runs: in the (still unused) shared-memory
    // row area when the row fits there, else in the global row scratch.
    unsigned long long* smemMask = reinterpret_cast<unsigned long long*>(smem);
    const int smemMaskRows = 2 * smemRows;
    auto mask = [&](int r) -> unsigned long long& { return r < smemMaskRows ? smemMask[r] : rowMask[r]; };
    int fIsl = 0, fRows = 0, fCons = 0, fMovers = 0;
    bool fast = false;
    if (coloured) {
        // the coloured solver's islands as connected components over the CTA: the table in shared
        // memory with the radix sort's work area at its end, else in the world's global table region
        // with the shared-memory area as the sort's work
        const int workBytes = RadixWorkInts() * (int)sizeof(int);
        unsigned char* sm = reinterpret_cast<unsigned char*>(smemBase);
        const int tableBytes = (smemBytes - workBytes) & ~15;
        if (sm && tableBytes > 0)
            fast = buildIslandsParallel<IslPacked>(sm, tableBytes, reinterpret_cast<int*>(sm + tableBytes),
                                                   sColourStart + 1, fIsl, fRows, fCons, fMovers);
        if (!fast)
            fast = buildIslandsParallel<IslWide>(islTab, d.islTabBytes,
                                                 sm && smemBytes >= workBytes ? reinterpret_cast<int*>(sm) : nullptr,
                                                 sColourStart + 1, fIsl, fRows, fCons, fMovers);
    }
    if (!fast)
        fast = buildIslandsTable<IslPacked>(reinterpret_cast<unsigned char*>(smemBase), smemBytes, coloured,
                                            sColourStart + 1, fIsl, fRows, fCons, fMovers);
    if (!fast)
        fast = buildIslandsTable<IslWide>(islTab, d.islTabBytes, coloured, sColourStart + 1, fIsl, fRows, fCons,
                                          fMovers);
    if (fast) {
        if (tid() == 0) {
            sIslands = fIsl;
            sRows = fRows;
            sCons = fCons;
            st->islands = fIsl;
            st->solvedBodies = fMovers;
            st->solvedContacts = fCons;
        }
    } else if (tid() == 0) {
        int nIsl = 0, bCur = 0, cCur = 0, jCur = 0, movers = 0;
        for (int seed = st->bodyList; seed != kNullIdx; seed = bj[seed].y) {
            int fl = bi[seed].y;
            if (fl & kBIsland) continue;
            if ((fl & kBAwake) == 0 || (fl & kBActive) == 0) continue;
            if (bi[seed].x == kStatic) continue;
            int bStart = bCur, cStart = cCur, jStart = jCur;
            int stackCount = 0;
            sStack[stackCount++] = seed;
            bi[seed].y = fl | kBIsland;
            while (stackCount > 0) {
                int b = sStack[--stackCount];
                if (bCur >= d.rowCap) { atomicOr(&st->error, kErrCapacity); stackCount = 0; break; }
                bj[b].z = bCur - bStart;
                if (coloured) mask(bCur) = 0ull;
                sBody[bCur++] = b;
                if (bi[b].x != kStatic) ++movers;
                setAwake(b, true);
                if (bi[b].x == kStatic) continue;
                B2G_WALK(e, bi[b].w, eNext(e), 2 * d.contactCap + 2) {
                    int c = e >> 1;
                    int4 info = ci[c];
                    if (info.x & kCIsland) continue;
                    if ((info.x & kCEnabled) == 0 || (info.x & kCTouching) == 0) continue;
                    if (fi[info.y].w != 0 || fi[info.z].w != 0) continue;
                    sContact[cCur++] = c;
                    ci[c].x = info.x | kCIsland;
                    int other = (e & 1) == 0 ? fixBody(info.z) : fixBody(info.y);
                    if (bi[other].y & kBIsland) continue;
                    sStack[stackCount++] = other;
                    bi[other].y |= kBIsland;
                }
                B2G_WALK(e, bj[b].x, jNext(e), 2 * d.jointCount + 2) {
                    Joint& J = jt[e >> 1];
                    if (J.islandFlag) continue;
                    int other = jOther(e);
                    if ((bi[other].y & kBActive) == 0) continue;
                    sJoint[jCur++] = e >> 1;
                    J.islandFlag = 1;
                    if (bi[other].y & kBIsland) continue;
                    sStack[stackCount++] = other;
                    bi[other].y |= kBIsland;
                }
            }
            islands[nIsl] = make_int4(bStart, bCur - bStart, cStart, cCur - cStart);
            islandJ[nIsl] = make_int2(jStart, jCur - jStart);
            ++nIsl;
            // Island-local body rows of this island's constraints, taken now: a static body can be
            // in several islands and its island index is overwritten by each island's DFS.
            for (int i = cStart; i < cCur; ++i) {
                int4 info = ci[sContact[i]];
                const int bA = fixBody(info.y), bB = fixBody(info.z);
                const int rA = bStart + bj[bA].z, rB = bStart + bj[bB].z;
                vc[i].idx = make_int4(rA, rB, 0, 0);
                if (coloured) {
                    // Greedy colouring in island order: the lowest colour used by neither dynamic
                    // body. Static and kinematic bodies take no impulse, so they constrain nothing.
                    const bool dA = bi[bA].x == kDynamic, dB = bi[bB].x == kDynamic;
                    const unsigned long long used = (dA ? mask(rA) : 0ull) | (dB ? mask(rB) : 0ull);
                    const unsigned long long freeBits = ~used & ((1ull << kSerialColour) - 1ull);
                    const int col = freeBits ? __ffsll((long long)freeBits) - 1 : kSerialColour;
                    if (col != kSerialColour) {
                        if (dA) mask(rA) |= 1ull << col;
                        if (dB) mask(rB) |= 1ull << col;
                    }
                    cColour[i] = col;
                    ++sColourStart[col + 1];
                }
            }
            for (int i = jStart; i < jCur; ++i) {
                Joint& J = jt[sJoint[i]];
                J.indexA = bStart + bj[J.bodyA].z;
                J.indexB = bStart + bj[J.bodyB].z;
                if (J.type == kJointGear) {
                    J.indexC = bStart + bj[J.bodyC].z;
                    J.indexD = bStart + bj[J.bodyD].z;
                }
            }
            for (int i = bStart; i < bCur; ++i)
                if (bi[sBody[i]].x == kStatic) bi[sBody[i]].y &= ~kBIsland;
        }
        sIslands = nIsl;
        sRows = bCur;
        sCons = cCur;
        st->islands = nIsl;
        st->solvedBodies = movers;
        st->solvedContacts = cCur;
    }
    __syncthreads();
    if (coloured) {
        // island contacts grouped by colour; the order inside a colour does not matter (its
        // constraints are independent) except in the serial bucket, which is kept in island order
        if (tid() == 0) {
            for (int k = 0; k < kColours; ++k) sColourStart[k + 1] += sColourStart[k];
            int used = 0;
            for (int k = 0; k < kSerialColour; ++k)
                if (sColourStart[k + 1] > sColourStart[k]) used = k + 1;
            st->colours = used + (sColourStart[kColours] > sColourStart[kSerialColour] ? 1 : 0);
        }
        for (int k = tid(); k < kColours; k += nthreads()) sColourCursor[k] = 0;
        __syncthreads();
        const int n = sCons;
        for (int i = tid(); i < n; i += nthreads()) {
            const int col = cColour[i];
            if (col == kSerialColour) continue;
            colourList[sColourStart[col] + atomicAdd(&sColourCursor[col], 1)] = i;
        }
        if (tid() == 0 && sColourStart[kColours] > sColourStart[kSerialColour]) {
            int w = sColourStart[kSerialColour];
            for (int i = 0; i < n; ++i)
                if (cColour[i] == kSerialColour) colourList[w++] = i;
        }
        __syncthreads();
    }
    unsigned long long t1 = clock64();
    const int nIsl = sIslands;
    solveIslands(P, nIsl, sRows, sCons, smem, smemRows, smemContacts, coloured ? sColourStart : nullptr);
    unsigned long long t2 = clock64();
    // A static body may sit in several islands; its awake flag ends as the last such island left it:
    // the largest island index per static body (sWake, free after the collide phase), then its flag.
    if (tid() == 0) {
        st->cyc[2] = t1 - tSolve0;
        st->cyc[3] = t2 - t1;
    }
    for (int b = tid(); b < nb; b += nthreads()) sWake[b] = -1;
    __syncthreads();
    for (int i = tid(); i < nIsl; i += nthreads()) {
        const int4 isl = islands[i];
        for (int k = isl.x; k < isl.x + isl.y; ++k) {
            const int b = sBody[k];
            if (bi[b].x == kStatic) atomicMax(&sWake[b], i);
        }
    }
    __syncthreads();
    for (int b = tid(); b < nb; b += nthreads()) {
        const int i = sWake[b];
        if (i < 0) continue;
        if (sleepOut[i]) bi[b].y &= ~kBAwake;
        else bi[b].y |= kBAwake;
    }
    if (treeLogId && tid() == 0) treeLog(0, make_float4(0.0f, 0.0f, 0.0f, 0.0f), kTreeStepMark);
    __syncthreads();
    for (int b = tid(); b < nb; b += nthreads()) {
        if ((bi[b].y & kBIsland) == 0 || bi[b].x == kStatic) continue;
        syncFixtures(b, nullptr, kTreeDiscrete);
    }
    __syncthreads();
    unsigned long long t3 = clock64();
    findNewContacts();
    if (tid() == 0) {
        st->cyc[4] = t3 - t2;
        st->cyc[5] = clock64() - t3;
    }
}

// ------------------------------------------------------------------ SolveTOI
// b2World::SolveTOI (Dynamics/b2World.cpp:579-896). One event at a time, as the reference: thread 0
// scans the contact list in order (mutating sweeps as the reference does), the time of impact of every
// contact that needs one is computed in parallel, thread 0 takes the earliest, and sub-steps it.
// The reset at the start of a completed step's continuous phase (b2World.cpp:583-599): island flags
// and sweep times of the bodies, TOI flags, counts and cached times of the contacts.
__device__ void Wd::resetToi()
{
    for (int b = tid(); b < d.bodyCount; b += nthreads()) {
        bi[b].y &= ~kBIsland;
        sw[b].w = 0.0f;
    }
    const int nc = st->contactCount;
    for (int k = tid(); k < nc; k += nthreads()) {
        int c = order[k];
        ci[c].x &= ~(kCToi | kCIsland);
        ci[c].w = 0;
        cp[c].w = 1.0f;
    }
}

// What the scan of b2World::SolveTOI (b2World.cpp:609-650) does with a contact whose ci record is
// info: 0 skipped (disabled,
// too many sub-steps, a sensor, no awake non-static body, or neither body a bullet, static or
// kinematic), 1 its cached time of impact, 2 a time of impact to compute.
__device__ int Wd::toiKind(const int4& info) const
{
    if ((info.x & kCEnabled) == 0 || info.w > kMaxSubSteps) return 0;
    if (info.x & kCToi) return 1;
    const int4 a = fi[info.y], b = fi[info.z];
    if (a.w != 0 || b.w != 0) return 0;
    const int4 iA = bi[a.x], iB = bi[b.x];
    const bool activeA = (iA.y & kBAwake) && iA.x != kStatic;
    const bool activeB = (iB.y & kBAwake) && iB.x != kStatic;
    const bool collideA = (iA.y & kBBullet) || iA.x != kDynamic;
    const bool collideB = (iB.y & kBBullet) || iB.x != kDynamic;
    return (activeA || activeB) && (collideA || collideB) ? 2 : 0;
}

// Tail indices per block of the earliest-event selection in Wd::solveTOI.
constexpr int kSelBlock = 256;

__device__ void Wd::solveTOI(const StepParams& P)
{
    __shared__ int sN, sDone, sMin;
    __shared__ float sMinAlpha;
    // ToiKernel may have done the reset and the first pass's times of impact already
    const bool prepared = st->toiPrepared != 0;
    if (st->stepComplete && !prepared) resetToi();
    __syncthreads();
    if (tid() == 0) st->toiPrepared = 0;
    __shared__ int sAdvance;
    __shared__ float sBestA[kMaxToiCta];
    __shared__ int sBestK[kMaxToiCta];
    unsigned long long tMark = clock64();
    auto stamp = [&](int slot) {
        if (tid() == 0) {
            const unsigned long long now = clock64();
            st->cyc[slot] += now - tMark;
            tMark = now;
        }
    };
    // The scan's outcome is kept per contact between events, indexed by the contact's position from
    // the list tail (vsep[t] = {alpha, or 2 when the scan skips it; contact slot}, cColour[c] = t):
    // no contact leaves the list during the continuous phase and new ones are prepended, so that
    // index is stable and list order is descending t. An event changes the outcome only of the
    // contacts it touches: the event contact, the contacts of the non-static bodies of its mini
    // island (invalidated, woken or moved) and the contacts it creates. Those (the dirty list in
    // colourList, deduplicated by the event stamp in evType) are the only ones classified again; the
    // first pass classifies the whole list. These scratch columns belong to the collide and solve
    // phases, which set them before use.
    __shared__ int sDirty, sNeed, sEvMoved;
    // blocks of the earliest-event selection whose minimum an event made stale (listed as they are
    // marked; more than kStaleCap: every block's flag is read instead), and the block count the
    // previous selection covered (blocks beyond it are new and always computed)
    constexpr int kStaleCap = 256;
    __shared__ int sStale[kStaleCap];
    __shared__ int sNStale, sNBlkPrev;
    if (tid() == 0) { sNStale = 0; sNBlkPrev = 0; }
    __shared__ int sSortT[kMaxToiCta * 2], sSortC[kMaxToiCta * 2];
    if (tid() == 0) sDirty = 0;
    for (int event = 0;; ++event) {
        const int n = st->contactCount;
        const int nTask = event == 0 ? n : sDirty;
        const int* task = event == 0 ? order : colourList;
        if (tid() == 0) { sAdvance = 0; sNeed = 0; }
        if (event > 0 && nTask > 1) {
            // dirty contacts into list order (descending tail index), for the sweep advances below
            if (nTask <= 2 * kMaxToiCta) {
                for (int i = tid(); i < nTask; i += nthreads()) {
                    const int c = colourList[i];
                    sSortC[i] = c;
                    sSortT[i] = cColour[c];
                }
                __syncthreads();
                for (int i = tid(); i < nTask; i += nthreads()) {
                    const int ti = sSortT[i];
                    int r = 0;
                    for (int j = 0; j < nTask; ++j) r += sSortT[j] > ti ? 1 : 0;
                    colourList[r] = sSortC[i];
                }
            } else if (tid() == 0) {
                for (int i = 1; i < nTask; ++i) {
                    const int x = colourList[i], tx = cColour[x];
                    int j = i - 1;
                    while (j >= 0 && cColour[colourList[j]] < tx) { colourList[j + 1] = colourList[j]; --j; }
                    colourList[j + 1] = x;
                }
            }
        }
        __syncthreads();
        // Classify the contacts in parallel: 0 skipped, 1 cached TOI, 2 TOI needed. Whether a
        // contact is skipped does not depend on the sweeps, so this is order-free. Each thread
        // gathers kBatch contacts one dependency level at a time (list slot, contact, its fixtures,
        // their bodies), so the global loads of a level overlap instead of queueing.
        constexpr int kBatch = 8;
        for (int k0 = tid(); k0 < nTask; k0 += kBatch * nthreads()) {
            int c[kBatch];
            int4 info[kBatch];
            int fA[kBatch], fB[kBatch];
            bool live[kBatch];
#pragma unroll
            for (int j = 0; j < kBatch; ++j) {
                const int k = k0 + j * nthreads();
                c[j] = k < nTask ? task[k] : -1;
            }
#pragma unroll
            for (int j = 0; j < kBatch; ++j) info[j] = c[j] >= 0 ? ci[c[j]] : make_int4(0, 0, 0, 0);
#pragma unroll
            for (int j = 0; j < kBatch; ++j) {
                live[j] = c[j] >= 0 && (info[j].x & kCEnabled) != 0 && info[j].w <= kMaxSubSteps &&
                          (info[j].x & kCToi) == 0;
                const int4 a = live[j] ? fi[info[j].y] : make_int4(0, 0, 0, 1);
                const int4 b = live[j] ? fi[info[j].z] : make_int4(0, 0, 0, 1);
                fA[j] = a.w == 0 && b.w == 0 ? a.x : -1;  // body of fixture A, -1 when a sensor
                fB[j] = b.x;
            }
#pragma unroll
            for (int j = 0; j < kBatch; ++j) {
                const int k = k0 + j * nthreads();
                if (c[j] < 0) continue;
                int kind = 0;
                if ((info[j].x & kCEnabled) != 0 && info[j].w <= kMaxSubSteps) {
                    if (info[j].x & kCToi) kind = 1;
                    else if (fA[j] >= 0) {
                        const int bA = fA[j], bB = fB[j];
                        const int4 iA = bi[bA], iB = bi[bB];
                        const bool activeA = (iA.y & kBAwake) && iA.x != kStatic;
                        const bool activeB = (iB.y & kBAwake) && iB.x != kStatic;
                        const bool collideA = (iA.y & kBBullet) || iA.x != kDynamic;
                        const bool collideB = (iB.y & kBBullet) || iB.x != kDynamic;
                        if ((activeA || activeB) && (collideA || collideB)) {
                            kind = 2;
                            if (sw[bA].w != sw[bB].w) sAdvance = 1;
                            sStatus[atomicAdd(&sNeed, 1)] = k;
                        }
                    }
                }
                TOITask& T = toi[k];
                T.contact = c[j];
                T.kind = kind;
            }
        }
        __syncthreads();
        if (sAdvance) {
            // Some pair has bodies at different sweep times: the reference advances the earlier body
            // while it scans, in list order, and later pairs see the advanced sweep. Replay on one
            // thread (contacts the scan skips or finds cached advance nothing).
            if (tid() == 0) {
                for (int k = 0; k < nTask; ++k) {
                    TOITask& T = toi[k];
                    if (T.kind != 2) continue;
                    int4 info = ci[T.contact];
                    int bA = fixBody(info.y), bB = fixBody(info.z);
                    Sweep sA = sweep(bA), sB = sweep(bB);
                    float alpha0 = sA.alpha0;
                    if (sA.alpha0 < sB.alpha0) {
                        alpha0 = sB.alpha0;
                        SweepAdvance(sA, alpha0);
                        setSweep(bA, sA);
                    } else if (sB.alpha0 < sA.alpha0) {
                        alpha0 = sA.alpha0;
                        SweepAdvance(sB, alpha0);
                        setSweep(bB, sB);
                    }
                    T.alpha0 = alpha0;
                    T.sa = sA;
                    T.sb = sB;
                }
            }
        } else {
            // All pairs agree on alpha0, so no sweep changes during the scan: snapshot in parallel.
            for (int k = tid(); k < nTask; k += nthreads()) {
                TOITask& T = toi[k];
                if (T.kind != 2) continue;
                int4 info = ci[T.contact];
                int bA = fixBody(info.y), bB = fixBody(info.z);
                T.sa = sweep(bA);
                T.sb = sweep(bB);
                T.alpha0 = T.sa.alpha0;
            }
        }
        __syncthreads();
        // the times of impact, over the compacted list of tasks that need one (sStatus, filled by
        // the classification in any order) so that every thread gets a share
        for (int i = tid(); i < sNeed; i += nthreads()) {
            TOITask& T = toi[sStatus[i]];
            int4 info = ci[T.contact];
            int state;
            float beta;
            TimeOfImpact(&state, &beta, ProxyOf(shape[info.y]), ProxyOf(shape[info.z]), T.sa, T.sb, 1.0f);
            float alpha = state == kToiTouching ? Minf(T.alpha0 + (1.0f - T.alpha0) * beta, 1.0f) : 1.0f;
            cp[T.contact].w = alpha;
            ci[T.contact].x = info.x | kCToi;
        }
        __syncthreads();
        // the outcomes by tail index (the first pass also numbers the list and clears the stamps)
        for (int k = tid(); k < nTask; k += nthreads()) {
            const TOITask& T = toi[k];
            const int c = T.contact;
            int t;
            if (event == 0) {
                t = n - 1 - k;
                cColour[c] = t;
                evType[c] = 0;
            } else {
                t = cColour[c];
                // its block's minimum is stale: flag it, and list it the first time
                const int bk = t / kSelBlock;
                if (atomicExch(reinterpret_cast<int*>(&vimpL[bk]) + 2, __float_as_int(1.0f)) == 0) {
                    const int slot = atomicAdd(&sNStale, 1);
                    if (slot < kStaleCap) sStale[slot] = bk;
                }
            }
            vsep[t] = make_float2(T.kind != 0 ? cp[c].w : 2.0f, __int_as_float(c));
        }
        __syncthreads();
        stamp(16);
        // Earliest TOI, first in list order among equals (the reference keeps the first alpha <
        // minAlpha): the argmin over (alpha, -t) of the outcomes with alpha < 1 (a later tail index
        // is earlier in the list, so it wins a tie). Two levels: the minimum of every block of
        // kSelBlock tail indices is kept in vimpL {alpha, t, stale} (free scratch in this phase) and
        // recomputed, one warp per block, only where an outcome changed; then the blocks' minima.
        {
            const int nBlk = (n + kSelBlock - 1) / kSelBlock;
            const int lane = tid() & 31, nWarps = nthreads() >> 5;
            const int nStale = sNStale, nPrev = sNBlkPrev;
            const bool full = event == 0 || nStale > kStaleCap;
            const int nWork = full ? nBlk : nStale + max(nBlk - nPrev, 0);
            for (int i = tid() >> 5; i < nWork; i += nWarps) {
                const int bk = full ? i : (i < nStale ? sStale[i] : nPrev + (i - nStale));
                if (full && event > 0 && vimpL[bk].z == 0.0f) continue;
                if (!full && i < nStale && bk >= nPrev) continue;  // a new block: computed below
                float ba = 1.0f;
                int bt = -1;
                for (int t = bk * kSelBlock + lane; t < min(n, (bk + 1) * kSelBlock); t += 32) {
                    const float alpha = vsep[t].x;
                    if (alpha < 1.0f && (bt < 0 || alpha < ba || (alpha == ba && t > bt))) { ba = alpha; bt = t; }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    const float oa = __shfl_down_sync(0xffffffffu, ba, o);
                    const int ot = __shfl_down_sync(0xffffffffu, bt, o);
                    if (ot >= 0 && (bt < 0 || oa < ba || (oa == ba && ot > bt))) { ba = oa; bt = ot; }
                }
                if (lane == 0) vimpL[bk] = make_float4(ba, __int_as_float(bt), 0.0f, 0.0f);
            }
            __syncthreads();
            float best = 1.0f;
            int bestT = -1;
            for (int bk = tid(); bk < nBlk; bk += nthreads()) {
                const float4 m = vimpL[bk];
                const int t = __float_as_int(m.y);
                if (t >= 0 && (bestT < 0 || m.x < best || (m.x == best && t > bestT))) { best = m.x; bestT = t; }
            }
            sBestA[tid()] = best;
            sBestK[tid()] = bestT;
        }
        __syncthreads();
        if (tid() == 0) {
            float minAlpha = 1.0f;
            int minT = -1;
            for (int t = 0; t < nthreads(); ++t) {
                if (sBestK[t] < 0) continue;
                if (sBestA[t] < minAlpha || (sBestA[t] == minAlpha && sBestK[t] > minT)) {
                    minAlpha = sBestA[t];
                    minT = sBestK[t];
                }
            }
            int minC = minT < 0 ? kNullIdx : __float_as_int(vsep[minT].y);
            sNStale = 0;
            sNBlkPrev = (n + kSelBlock - 1) / kSelBlock;
            sMin = minC;
            sMinAlpha = minAlpha;
            sDone = 0;
            if (minC == kNullIdx || 1.0f - 10.0f * kEpsilon < minAlpha) {
                st->stepComplete = 1;
                sDone = 1;
            } else if (event >= P.maxToiEvents) {
                atomicOr(&st->error, kErrTimeout);
                st->stepComplete = 1;
                sDone = 1;
            }
        }
        __syncthreads();
        stamp(17);
        if (sDone) break;
        if (tid() == 0) {
            st->toiEvents = event + 1;
            sDirty = 0;
            int nMovedEv = 0;  // proxies the event's fixture synchronisation moves (listed in movedList)
            const int mc = sMin;
            const float minAlpha = sMinAlpha;
            int4 info = ci[mc];
            int bA = fixBody(info.y), bB = fixBody(info.z);
            Sweep backup1 = sweep(bA), backup2 = sweep(bB);
            advance(bA, minAlpha);
            advance(bB, minAlpha);
            {
                const int before = ci[mc].x;
                update(mc);
                if (evLog)
                    appendUpdateEvents(mc, updateEventBits((before & kCTouching) != 0, (ci[mc].x & kCTouching) != 0,
                                                           fi[ci[mc].y].w != 0 || fi[ci[mc].z].w != 0));
            }
            ci[mc].x &= ~kCToi;
            ci[mc].w += 1;
            int fl = ci[mc].x;
            bool skip = false;
            if ((fl & kCEnabled) == 0 || (fl & kCTouching) == 0) {
                ci[mc].x = fl & ~kCEnabled;
                setSweep(bA, backup1);
                setSweep(bB, backup2);
                syncTransform(bA);
                syncTransform(bB);
                skip = true;
            }
            if (!skip) {
                // island bodies (bit = island position) this event woke: a woken kinematic body's
                // contacts join the dirty list below (an awake one's cannot change their outcome)
                static_assert(2 * kMaxTOIContacts <= 64, "one bit per mini-island body");
                unsigned long long woke = 0ull;
                if ((bi[bA].y & kBAwake) == 0) woke |= 1ull;
                if ((bi[bB].y & kBAwake) == 0) woke |= 2ull;
                setAwake(bA, true);
                setAwake(bB, true);
                // mini island in the scratch rows (b2World.cpp:700-780)
                int nBodies = 0, nContacts = 0;
                const int bodyCap = 2 * kMaxTOIContacts, contactCap = kMaxTOIContacts;
                bj[bA].z = nBodies; sBody[nBodies++] = bA;
                bj[bB].z = nBodies; sBody[nBodies++] = bB;
                sContact[nContacts++] = mc;
                bi[bA].y |= kBIsland;
                bi[bB].y |= kBIsland;
                ci[mc].x |= kCIsland;
                int pairB[2] = {bA, bB};
                for (int kk = 0; kk < 2; ++kk) {
                    int body = pairB[kk];
                    if (bi[body].x != kDynamic) continue;
                    B2G_WALK(e, bi[body].w, eNext(e), 2 * d.contactCap + 2) {
                        if (nBodies == bodyCap) break;
                        if (nContacts == contactCap) break;
                        int c = e >> 1;
                        int4 ic = ci[c];
                        if (ic.x & kCIsland) continue;
                        int other = (e & 1) == 0 ? fixBody(ic.z) : fixBody(ic.y);
                        if (bi[other].x == kDynamic && (bi[body].y & kBBullet) == 0 && (bi[other].y & kBBullet) == 0)
                            continue;
                        if (fi[ic.y].w != 0 || fi[ic.z].w != 0) continue;
                        Sweep backup = sweep(other);
                        if ((bi[other].y & kBIsland) == 0) advance(other, minAlpha);
                        update(c);
                        if (evLog)
                            appendUpdateEvents(c, updateEventBits((ic.x & kCTouching) != 0, (ci[c].x & kCTouching) != 0,
                                                                  fi[ic.y].w != 0 || fi[ic.z].w != 0));
                        int fc = ci[c].x;
                        if ((fc & kCEnabled) == 0 || (fc & kCTouching) == 0) {
                            setSweep(other, backup);
                            syncTransform(other);
                            continue;
                        }
                        ci[c].x = fc | kCIsland;
                        sContact[nContacts++] = c;
                        if (bi[other].y & kBIsland) continue;
                        bi[other].y |= kBIsland;
                        if (bi[other].x != kStatic) {
                            if ((bi[other].y & kBAwake) == 0) woke |= 1ull << nBodies;
                            setAwake(other, true);
                        }
                        bj[other].z = nBodies;
                        sBody[nBodies++] = other;
                    }
                }
                stamp(18);
                // b2Island::SolveTOI (Dynamics/b2Island.cpp:386-485). The mini island's rows and
                // constraint records live in shared memory when they fit (the CTA's dynamic shared
                // memory is free during the continuous phase), else in the global scratch.
                const int miniBytes = (2 * bodyCap) * (int)sizeof(float4) +
                                      kMaxTOIContacts * (int)(sizeof(VelConstraint) + sizeof(PosConstraint) + sizeof(float4));
                const bool miniShared = miniBytes <= smemBytes;
                float4* mPos = miniShared ? smemBase : sPos;
                float4* mVel = miniShared ? smemBase + bodyCap : sVel;
                VelConstraint* mVc = miniShared ? reinterpret_cast<VelConstraint*>(smemBase + 2 * bodyCap) : vc;
                PosConstraint* mPc = miniShared ? reinterpret_cast<PosConstraint*>(mVc + kMaxTOIContacts) : pc;
                float4* mImp = miniShared ? reinterpret_cast<float4*>(mPc + kMaxTOIContacts) : vimp;
                float subDt = (1.0f - minAlpha) * P.dt;
                for (int i = 0; i < nBodies; ++i) {
                    int b = sBody[i];
                    float4 s = sw[b], v = vel[b];
                    mPos[i] = make_float4(s.x, s.y, s.z, 0.0f);
                    mVel[i] = make_float4(v.x, v.y, v.z, 0.0f);
                }
                // rows 0..nBodies-1 of the scratch hold the mini island (island index == row)
                for (int i = 0; i < nContacts; ++i) {
                    int4 ic = ci[sContact[i]];
                    VelConstraint v;
                    v.idx = make_int4(bj[fixBody(ic.y)].z, bj[fixBody(ic.z)].z, 0, 0);
                    PosConstraint p;
                    float4 im;
                    ContactSetup(*this, v, p, im, sContact[i], false, 1.0f);
                    mVc[i] = v;
                    mPc[i] = p;
                    mImp[i] = im;
                }
                const int toiA = bj[bA].z, toiB = bj[bB].z;
                for (int it = 0; it < 20; ++it)
                    if (SweepPosition(mPc, 0, nContacts, mPos, true, toiA, toiB)) break;
                {
                    float4 pA = mPos[toiA], pB = mPos[toiB];
                    float4 a0 = sw0[bA];
                    sw0[bA] = make_float4(pA.x, pA.y, pA.z, a0.w);
                    float4 b0 = sw0[bB];
                    sw0[bB] = make_float4(pB.x, pB.y, pB.z, b0.w);
                }
                for (int i = 0; i < nContacts; ++i) ContactInitVelocity(*this, mVc[i], mPc[i], mPos, mVel);
                for (int it = 0; it < P.velocityIterations; ++it) SweepVelocity(mVc, mImp, 0, nContacts, mVel);
                const float h = subDt;
                for (int i = 0; i < nBodies; ++i) {
                    float4 p4 = mPos[i], v4 = mVel[i];
                    IntegratePosition(p4, v4, h);
                    mPos[i] = p4;
                    mVel[i] = v4;
                    int b = sBody[i];
                    sw[b] = make_float4(p4.x, p4.y, p4.z, sw[b].w);
                    vel[b] = make_float4(v4.x, v4.y, v4.z, 0.0f);
                    syncTransform(b);
                }
                // b2Island::Report of the sub-step island (b2Island.cpp:515): PostSolve with the TOI
                // velocity impulses, which are not stored in the manifolds
                if (evLog)
                    for (int i = 0; i < nContacts; ++i) {
                        const int4 ic = ci[sContact[i]];
                        const float4 im = mImp[i];
                        const int pcn = mVc[i].idx.z;
                        putEvent(st->eventCount++, kEvPostSolve, ic.y, ic.z, pcn, pcn > 0 ? im.x : 0.0f,
                                 pcn > 1 ? im.z : 0.0f, pcn > 0 ? im.y : 0.0f, pcn > 1 ? im.w : 0.0f);
                    }
                stamp(19);
                // dynamic bodies: fixtures synchronised, contacts' TOIs invalidated; the contacts of
                // every dynamic island body and of every kinematic one this event woke join the dirty
                // list
                for (int i = 0; i < nBodies; ++i) {
                    int b = sBody[i];
                    bi[b].y &= ~kBIsland;
                    if (bi[b].x == kStatic) continue;
                    const bool dynamic = bi[b].x == kDynamic;
                    if (dynamic) syncFixtures(b, &nMovedEv);
                    else if (((woke >> i) & 1ull) == 0ull) continue;
                    B2G_WALK(e, bi[b].w, eNext(e), 2 * d.contactCap + 2) {
                        const int c = e >> 1;
                        if (dynamic) ci[c].x &= ~(kCToi | kCIsland);
                        if (evType[c] != event + 1) {
                            evType[c] = event + 1;
                            colourList[sDirty++] = c;
                        }
                    }
                }
            }
            if (evType[mc] != event + 1) {
                evType[mc] = event + 1;
                colourList[sDirty++] = mc;
            }
            sDone = skip ? 2 : 0;
            sEvMoved = nMovedEv;
        }
        __syncthreads();
        stamp(20);
        if (sDone == 2) continue;
        findNewContacts(true, sEvMoved);
        __syncthreads();
        {
            // the contacts the event created sit at the head of the list
            const int n2 = st->contactCount, nNew = n2 - n, base = sDirty;
            for (int k = tid(); k < nNew; k += nthreads()) {
                const int c = order[k];
                cColour[c] = n2 - 1 - k;
                evType[c] = event + 1;
                colourList[base + k] = c;
            }
            __syncthreads();
            if (tid() == 0) sDirty = base + nNew;
        }
        stamp(21);
        if (st->subStepping) {
            if (tid() == 0) st->stepComplete = 0;
            __syncthreads();
            break;
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ kernels
// One step of a batch is, in stream order:
//   NarrowphaseKernel  (flat, every contact row of the class's worlds) per-step counters reset;
//                      manifolds of the collide phase evaluated ahead
//   StepKernel         (per world, per launch class) new-fixture pairs, collide (commits the staged
//                      manifolds), island solve, fixture sync and pair finding
//   ToiKernel          (flat, every body and contact row of the class's worlds) the continuous
//                      phase's reset and the first pass of times of impact
//   StepToiKernel      (per world, per launch class) the continuous phase's event loop, force clearing
// The flat pre-passes compute, per contact and in any order, values the reference computes while it
// walks the contact list; the per-world kernels consume them in list order, so the results are the
// reference's bit for bit. One thread per contact row keeps every SM busy with short independent
// work (most rows are spare capacity and return at once), where the per-world kernels hold a
// world's sequential phases. Each class launches only its own worlds' rows: chunks of kRowChunk rows
// of one world, listed in schedule order (bench batch, one call: the two pre-pass stages 0.19 + 0.27
// ms with full-batch grids gated by class, 0.16 + 0.22 ms with the chunks).

// Per-step counters of the world, zeroed before the step (profile slots included).
__device__ void ResetStepCounters(WorldState* st)
{
    st->toiEvents = 0;
    st->islands = 0;
    st->solvedBodies = 0;
    st->solvedContacts = 0;
    st->pairsFound = 0;
    st->colours = 0;
    st->velIters = 0;
    st->residual = 0.0f;
    st->warmLearned = 0;
    st->velItersSum = 0;
    st->maxPenetration = 0.0f;
    st->eventCount = 0;
    st->eventsDropped = 0;
    for (int i = 0; i < kProfileSlots; ++i) st->cyc[i] = 0;
}

// The evaluations of b2ContactManager::Collide (Dynamics/b2ContactManager.cpp:107-172), ahead of the
// step, one thread per contact row of the class's worlds: the k-th live contact of a world's list, if
// it is a non-sensor contact with an awake non-static body whose fat AABBs overlap, gets the manifold
// b2Contact::Update would compute (evaluation at the current transforms, impulses matched by id) in
// its stage record. Nothing the collide phase does before it updates a contact changes those
// inputs, so the collide phase commits the record when it reaches the contact; contacts left out
// (tag 0: asleep, sensors, apart) it evaluates itself. Worlds with new fixtures create contacts
// before their collide phase and are left out whole. Row 0 of each world resets its counters.
// chunks: one per CTA, {world, first contact index, contacts, 0} (kRowChunk rows at most).
__global__ void __launch_bounds__(kRowChunk) NarrowphaseKernel(Batch B, const int4* chunks)
{
    const int4 ch = chunks[blockIdx.x];
    if ((int)threadIdx.x >= ch.z) return;
    const int w = ch.x;
    WorldState* st = B.state + w;
    const int k = ch.y + (int)threadIdx.x;
    const bool newFixture = st->newFixture != 0;
    if (k == 0) {
        ResetStepCounters(st);
        st->staged = newFixture ? 0 : 1;
    }
    if (newFixture || k >= st->contactCount) return;
    Wd W;
    W.init(B, w);
    const int c = W.order[k];
    const int4 info = W.ci[c];
    const int4 a = W.fi[info.y], b = W.fi[info.z];
    int tag = 0;
    if (a.w == 0 && b.w == 0) {
        const bool activeA = W.type(a.x) != kStatic && W.awake(a.x);
        const bool activeB = W.type(b.x) != kStatic && W.awake(b.x);
        if ((activeA || activeB) && Overlap(W.fat[a.z], W.fat[b.z])) {
            Manifold m;
            W.evaluateManifold(c, m, nullptr);
            W.writeStage(c, m);
            tag = 1;
        }
    }
    W.stageOf(c)->tag = tag;
}

// b2World::Step (Dynamics/b2World.cpp:899-963) for world schedule[blockIdx.x], one CTA per world, up
// to the continuous phase: new-fixture pairs, collide, island solve (with fixture synchronisation and
// pair finding at its end).
// Shared memory (its size is the launch's choice, LaunchShape) stages the island body rows
// (positions, then velocities) and the accumulated impulses of the island contacts when a world's
// fit, and the broadphase proxies, pair keys and list heads outside the island solve; every use
// falls back to global memory when the world is larger, so the shape changes speed, never results.
// Register caps: StepKernel 128 registers (CTAs of up to 512 threads, the width single large worlds
// use; 2 resident CTAs of 256 = 4 of 128), StepToiKernel 168 (at most 64 threads, 6 resident; its
// time-of-impact code spills more when capped lower). Measured on the bench batch with 128-thread
// CTAs at most: StepKernel/StepToiKernel resident CTAs 4/3 3.89 ms per step coloured, 10.20 plain;
// 3/3 4.05, 10.51; 4/4 4.01, 10.33; 5/4 4.24, 11.37 (fewer registers spill).
__global__ void __launch_bounds__(kMaxCta, 1) StepKernel(Batch B, StepParams P, const int* schedule, LaunchShape L)
{
    extern __shared__ float4 smem[];
    Wd W;
    W.init(B, schedule ? schedule[blockIdx.x] : blockIdx.x);
    W.smemBase = smem;
    W.smemBytes = (2 * L.smemRows + L.smemContacts) * (int)sizeof(float4);
    const unsigned long long t0 = clock64();
    unsigned long long t1 = t0, t2 = t0;
    if (P.phase != 2) {
        const bool newFixture = W.st->newFixture != 0;
        __syncthreads();
        if (tid() == 0) W.st->newFixture = 0;
        if (newFixture) W.findNewContacts();
        __syncthreads();
        t1 = clock64();
        W.collide();
        t2 = clock64();
    }
    if (P.phase != 1 && W.st->stepComplete && P.dt > 0.0f) W.solve(P, smem, L.smemRows, L.smemContacts);
    __syncthreads();
    if (tid() == 0) {
        const unsigned long long t3 = clock64();
        if (P.phase != 2) {
            W.st->cyc[0] = t1 - t0;
            W.st->cyc[1] = t2 - t1;
            W.st->cyc[7] = t3 - t0;
        } else {
            W.st->cyc[7] += t3 - t0;
        }
    }
}

// Verdicts of the user contact filter written into the table: keys[i] -> vals[i], one thread per
// verdict (the keys were inserted by the step that met them).
__global__ void FilterVerdictKernel(Batch B, const unsigned long long* keys, const int* vals, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long key = keys[i];
    unsigned slot = FilterSlot(key, B.filterCap);
    for (int probe = 0; probe < B.filterCap; ++probe, slot = (slot + 1) & (unsigned)(B.filterCap - 1)) {
        if (B.filterKeys[slot] == key) { B.filterVals[slot] = vals[i]; return; }
        if (B.filterKeys[slot] == ~0ull) return;
    }
}

// Contact changes between the halves of a split step (b2Contact::SetEnabled, SetFriction,
// SetRestitution, SetTangentSpeed made by a PreSolve listener), in order, one thread.
__global__ void ContactEditKernel(Batch B, const ContactEdit* edits, int n)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int i = 0; i < n; ++i) {
        const ContactEdit e = edits[i];
        if (e.world < 0 || e.world >= B.worlds) continue;
        Wd W;
        W.init(B, e.world);
        if (e.contact < 0 || e.contact >= W.st->contactCount) continue;
        const int c = W.order[e.contact];
        if (e.flags & 1) W.ci[c].x = e.enabled ? (W.ci[c].x | kCEnabled) : (W.ci[c].x & ~kCEnabled);
        float4 p = W.cp[c];
        if (e.flags & 2) p.x = e.friction;
        if (e.flags & 4) p.y = e.restitution;
        if (e.flags & 8) p.z = e.tangentSpeed;
        W.cp[c] = p;
    }
}

// The first pass of b2World::SolveTOI (Dynamics/b2World.cpp:579-680) after a completed step, one
// thread per body row and per contact row of the class's worlds: the reset (body island flags and sweep
// times, contact TOI flags, counts and cached times), then for every contact the scan would compute
// a time of impact for, that time, cached on the contact as the scan caches it. After the reset every
// sweep starts at alpha0 = 0 (a contact thread takes that value instead of waiting for its bodies'
// reset), so the scan advances no sweep and each time of impact depends on its contact alone.
// StepToiKernel's event loop then finds them cached. The body-flag bits the classification reads
// (type, awake, bullet) are not the ones the reset clears.
// chunks: one per CTA, {world, first row, rows, 0 for body rows / 1 for contact rows}.
__global__ void __launch_bounds__(kRowChunk, 4) ToiKernel(Batch B, float dt, const int4* chunks)
{
    const int4 ch = chunks[blockIdx.x];
    if ((int)threadIdx.x >= ch.z) return;
    const int w = ch.x;
    WorldState* st = B.state + w;
    if (!(st->continuous && dt > 0.0f && st->stepComplete)) return;
    if (ch.w == 0) {
        const int b = ch.y + (int)threadIdx.x;
        if (b == 0) st->toiPrepared = 1;
        if (b < B.desc[w].bodyCount) {
            const int r = B.desc[w].bodyBase + b;
            B.bi[r].y &= ~kBIsland;
            B.sw[r].w = 0.0f;
        }
        return;
    }
    const int k = ch.y + (int)threadIdx.x;
    if (k >= st->contactCount) return;
    Wd W;
    W.init(B, w);
    const int c = W.order[k];
    int4 info = W.ci[c];
    info.x &= ~(kCToi | kCIsland);
    info.w = 0;
    float alpha = 1.0f;
    if (W.toiKind(info) == 2) {
        Sweep sA = W.sweep(W.fixBody(info.y)), sB = W.sweep(W.fixBody(info.z));
        sA.alpha0 = 0.0f;
        sB.alpha0 = 0.0f;
        const float alpha0 = sA.alpha0;
        int state;
        float beta;
        TimeOfImpact(&state, &beta, ProxyOf(W.shape[info.y]), ProxyOf(W.shape[info.z]), sA, sB, 1.0f);
        alpha = state == kToiTouching ? Minf(alpha0 + (1.0f - alpha0) * beta, 1.0f) : 1.0f;
        info.x |= kCToi;
    }
    W.cp[c].w = alpha;
    W.ci[c] = info;
}

// The continuous phase of b2World::Step (b2World.cpp:948-958) and the end of the step: the TOI
// event loop, force clearing, inv_dt0.
// 168 registers: 6 resident CTAs of 64 threads, or 3 of 128 (the single-world form)
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 384 / kThreads) StepToiKernel(Batch B, StepParams P, const int* schedule,
                                                                      LaunchShape L)
{
    extern __shared__ float4 smem[];
    Wd W;
    W.init(B, schedule ? schedule[blockIdx.x] : blockIdx.x);
    W.smemBase = smem;
    W.smemBytes = (2 * L.smemRows + L.smemContacts) * (int)sizeof(float4);
    const unsigned long long t0 = clock64();
    if (W.st->continuous && P.dt > 0.0f) W.solveTOI(P);
    __syncthreads();
    if (W.st->clearForces)
        for (int b = tid(); b < W.d.bodyCount; b += nthreads()) W.frc[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (tid() == 0) {
        if (P.dt > 0.0f) W.st->inv_dt0 = 1.0f / P.dt;
        const unsigned long long t1 = clock64();
        W.st->cyc[6] = t1 - t0;
        W.st->cyc[7] += t1 - t0;
    }
}

// gb_body_edits: the edits in array order on one thread (they may repeat a body, and their order
// is the caller's call order).
__global__ void BodyEditKernel(Batch B, const BodyEdit* edits, int n)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int i = 0; i < n; ++i) {
        const BodyEdit e = edits[i];
        Wd W;
        W.init(B, e.world);
        W.applyEdit(e);
    }
}

} // namespace b2g

// Launch entries used by the host runtime (b2g_api.cu). A step is b2gLaunchNarrowphase, then
// b2gLaunchStep for every launch class, then b2gLaunchToi, then b2gLaunchStepToi for every class.
cudaError_t b2gLaunchNarrowphase(const b2g::Batch& B, const int4* chunks, int n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::NarrowphaseKernel<<<n, b2g::kRowChunk, 0, stream>>>(B, chunks);
    return cudaGetLastError();
}

cudaError_t b2gLaunchFilterVerdicts(const b2g::Batch& B, const unsigned long long* keys, const int* vals, int n,
                                    cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::FilterVerdictKernel<<<(n + 127) / 128, 128, 0, stream>>>(B, keys, vals, n);
    return cudaGetLastError();
}

cudaError_t b2gLaunchContactEdits(const b2g::Batch& B, const b2g::ContactEdit* edits, int n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::ContactEditKernel<<<1, 32, 0, stream>>>(B, edits, n);
    return cudaGetLastError();
}

cudaError_t b2gLaunchBodyEdits(const b2g::Batch& B, const b2g::BodyEdit* edits, int n, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::BodyEditKernel<<<1, 32, 0, stream>>>(B, edits, n);
    return cudaGetLastError();
}

cudaError_t b2gLaunchToi(const b2g::Batch& B, const b2g::StepParams& P, const int4* chunks, int n, cudaStream_t stream)
{
    if (!(P.dt > 0.0f) || n <= 0) return cudaSuccess;
    b2g::ToiKernel<<<n, b2g::kRowChunk, 0, stream>>>(B, P.dt, chunks);
    return cudaGetLastError();
}

static b2g::LaunchShape Shape(int smemRows, int smemContacts)
{
    b2g::LaunchShape L;
    L.smemRows = smemRows;
    L.smemContacts = smemContacts;
    return L;
}

cudaError_t b2gLaunchStep(const b2g::Batch& B, const b2g::StepParams& P, const int* schedule, int first, int count,
                          int threads, int smemRows, int smemContacts, cudaStream_t stream)
{
    if (count <= 0) return cudaSuccess;
    const size_t smem = (2 * (size_t)smemRows + smemContacts) * sizeof(float4);
    b2g::StepKernel<<<count, threads, smem, stream>>>(B, P, schedule + first, Shape(smemRows, smemContacts));
    return cudaGetLastError();
}

cudaError_t b2gLaunchStepToi(const b2g::Batch& B, const b2g::StepParams& P, const int* schedule, int first, int count,
                             int threads, int smemRows, int smemContacts, cudaStream_t stream)
{
    if (count <= 0) return cudaSuccess;
    const size_t smem = (2 * (size_t)smemRows + smemContacts) * sizeof(float4);
    // the continuous phase is mostly one thread's event loop: CTAs of at most kBatchToiCta threads,
    // or kMaxToiCta for a class of one world
    if (count == 1 && threads >= b2g::kMaxToiCta)
        b2g::StepToiKernel<b2g::kMaxToiCta><<<1, b2g::kMaxToiCta, smem, stream>>>(B, P, schedule + first,
                                                                                Shape(smemRows, smemContacts));
    else
        b2g::StepToiKernel<b2g::kBatchToiCta><<<count, threads < b2g::kBatchToiCta ? threads : b2g::kBatchToiCta, smem,
                                                 stream>>>(B, P, schedule + first, Shape(smemRows, smemContacts));
    return cudaGetLastError();
}
