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
    int* order;
    int* cnext;
    Joint* jt;
    int *sBody, *sStack, *sWake;
    float4 *sPos, *sVel;
    int *sContact, *sStatus;
    VelConstraint* vc;
    PosConstraint* pc;
    TOITask* toi;
    int4* islands;
    int2* islandJ;
    int* sJoint;
    int* sleepOut;
    unsigned long long* pairs;
    int* pairKeep;
    int* movedList;

    __device__ void init(const Batch& B, int w)
    {
        d = B.desc[w];
        st = B.state + w;
        int b = d.bodyBase, f = d.fixBase, p = d.proxyBase, c = d.contactBase, j = d.jointBase, q = d.pairBase;
        xf = B.xf + b; sw = B.sw + b; sw0 = B.sw0 + b; vel = B.vel + b; frc = B.frc + b; mas = B.mas + b;
        prop = B.prop + b; bi = B.bi + b; bj = B.bj + b;
        fi = B.fi + f; fm = B.fm + f; ff = B.ff + f; faabb = B.faabb + f; shape = B.shape + f;
        fat = B.fat + p; pfix = B.pfix + p; moved = B.moved + p; movedList = B.movedList + p;
        ci = B.ci + c; ce = B.ce + c; cp = B.cp + c; mh = B.mh + c; mv = B.mv + c; mp0 = B.mp0 + c; mp1 = B.mp1 + c;
        order = B.order + c; cnext = B.cnext + c;
        jt = B.joint + j; sJoint = B.sJoint + j;
        sBody = B.sBody + d.rowBase; sPos = B.sPos + d.rowBase; sVel = B.sVel + d.rowBase;
        sStack = B.sStack + b; sWake = B.sWake + b;
        islands = B.islands + b; islandJ = B.islandJ + b; sleepOut = B.sleepOut + b;
        sContact = B.sContact + c; sStatus = B.sStatus + c; vc = B.vc + c; pc = B.pc + c; toi = B.toi + c;
        pairs = B.pairs + q; pairKeep = B.pairKeep + q;
    }

    // ---------------------------------------------------------------- body helpers
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
    __device__ bool filterCollide(int fA, int fB) const
    {
        int4 a = ff[fA], b = ff[fB];
        if (a.z == b.z && a.z != 0) return a.z > 0;
        return (a.y & b.x) != 0 && (a.x & b.y) != 0;
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

    // b2Contact::Update (Dynamics/Contacts/b2Contact.cpp:164-245). Returns true when the touching
    // state of a non-sensor contact changed (the caller wakes both bodies).
    __device__ bool update(int c)
    {
        int4 info = ci[c];
        int fl = info.x | kCEnabled;
        bool wasTouching = (fl & kCTouching) != 0;
        int fA = info.y, fB = info.z;
        bool sensor = fi[fA].w != 0 || fi[fB].w != 0;
        int bA = fixBody(fA), bB = fixBody(fB);
        Xf xfA = xform(bA), xfB = xform(bB);
        bool touching;
        bool changed = false;
        if (sensor) {
            Proxy pa = ProxyOf(shape[fA]), pb = ProxyOf(shape[fB]);
            SimplexCache cache;
            cache.count = 0;
            cache.metric = 0.0f;
            Vec2 a, b;
            touching = Distance(&a, &b, &cache, pa, xfA, pb, xfB, true) < 10.0f * kEpsilon;
            mh[c].y = 0;
        } else {
            Manifold old;
            loadManifold(c, old);
            Manifold m;
            m.count = 0;
            m.type = old.type;
            m.localNormal = old.localNormal;
            m.localPoint = old.localPoint;
            Evaluate(&m, shape[fA], xfA, shape[fB], xfB);
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
            storeManifold(c, m);
            touching = m.count > 0;
            changed = touching != wasTouching;
        }
        if (touching) fl |= kCTouching;
        else fl &= ~kCTouching;
        ci[c].x = fl;
        return changed;
    }

    // ---------------------------------------------------------------- broadphase
    // b2Fixture::Synchronize + b2DynamicTree::MoveProxy (b2Fixture.cpp:154-177, b2DynamicTree.cpp:133-177)
    __device__ void syncFixtures(int b)
    {
        float4 s0 = sw0[b], m = mas[b];
        Xf xf1;
        xf1.q = RotOf(s0.z);
        xf1.p = V(s0.x, s0.y) - Mul(xf1.q, V(m.z, m.w));
        Xf xf2 = xform(b);
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
            moved[pid] = 1;
        }
    }

    // Contact factory order (Dynamics/Contacts/b2Contact.cpp:40-100): primary type pairs keep (A, B).
    __device__ static bool primaryOrder(int t1, int t2) { return t1 == t2 || (t1 == kPolygon && t2 == kCircle) || t1 == kEdge; }

    // b2ContactManager::FindNewContacts -> b2BroadPhase::UpdatePairs -> AddPair, CTA-wide.
    __device__ void findNewContacts();
    __device__ void collide();
    __device__ void solve(const StepParams& P);
    __device__ void solveTOI(const StepParams& P);
    __device__ void destroyContact(int c);
    __device__ void islandSolve(int island, const StepParams& P, float dt, float dtRatio);
};

// ------------------------------------------------------------------ CTA helpers
__device__ inline int tid() { return threadIdx.x; }
__device__ inline int nthreads() { return blockDim.x; }

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

// ------------------------------------------------------------------ FindNewContacts
__device__ void Wd::findNewContacts()
{
    __shared__ int sMoved, sPairs, sNew;
    if (tid() == 0) { sMoved = 0; sPairs = 0; sNew = 0; }
    __syncthreads();
    const int np = d.proxyCap;
    for (int p = tid(); p < np; p += nthreads())
        if (moved[p]) movedList[atomicAdd(&sMoved, 1)] = p;
    __syncthreads();
    const int m = sMoved;
    // Query every moved proxy's fat AABB against all proxies (b2BroadPhase.h:188-217); a pair whose
    // both proxies moved is emitted once, from the lower proxy id.
    const long long total = (long long)m * np;
    for (long long idx = tid(); idx < total; idx += nthreads()) {
        int q = movedList[idx / np];
        int p = (int)(idx % np);
        if (p == q || pfix[p] < 0) continue;
        if (moved[p] && p < q) continue;
        if (!Overlap(fat[p], fat[q])) continue;
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
    ctaSortKeys(pairs, n, d.pairCap);
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
    // Create in sorted pair order; each new contact goes to the front of every list
    // (b2ContactManager.cpp:229-293).
    if (tid() == 0) {
        int created = 0;
        for (int k = 0; k < n; ++k) {
            if (!pairKeep[k]) continue;
            int pA = (int)(pairs[k] >> 32), pB = (int)(pairs[k] & 0xffffffffu);
            int fa = pfix[pA], fb = pfix[pB];
            if (!primaryOrder(shape[fa].type, shape[fb].type)) { int t = fa; fa = fb; fb = t; }
            int c = st->freeContact;
            if (c == kNullIdx) { atomicOr(&st->error, kErrCapacity); break; }
            st->freeContact = cnext[c];
            float4 ma = fm[fa], mb = fm[fb];
            ci[c] = make_int4(kCEnabled, fa, fb, 0);
            cp[c] = make_float4(sqrtf(ma.x * mb.x), ma.y > mb.y ? ma.y : mb.y, 0.0f, 1.0f);
            mh[c] = make_int4(0, 0, 0, 0);
            mv[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            mp0[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            mp1[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            int bA = fixBody(fa), bB = fixBody(fb);
            int eA = 2 * c, eB = 2 * c + 1;
            int hA = bi[bA].w;
            ce[c] = make_int4(kNullIdx, hA, kNullIdx, kNullIdx);
            if (hA != kNullIdx) *ePrevP(hA) = eA;
            bi[bA].w = eA;
            int hB = bi[bB].w;
            ce[c].w = hB;
            if (hB != kNullIdx) *ePrevP(hB) = eB;
            bi[bB].w = eB;
            if (fi[fa].w == 0 && fi[fb].w == 0) {
                setAwake(bA, true);
                setAwake(bB, true);
            }
            sContact[created++] = c;
        }
        sNew = created;
    }
    __syncthreads();
    // order = reverse(new) ++ order
    int created = sNew;
    if (created > 0) {
        int live = st->contactCount;
        if (tid() == 0) {
            for (int i = live - 1; i >= 0; --i) order[i + created] = order[i];
            for (int i = 0; i < created; ++i) order[created - 1 - i] = sContact[i];
            st->contactCount = live + created;
        }
    }
    for (int i = tid(); i < m; i += nthreads()) moved[movedList[i]] = 0;
    __syncthreads();
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
    for (int b = tid(); b < d.bodyCount; b += nthreads()) sWake[b] = awake(b) ? -1 : INT_MAX;
    for (int k = tid(); k < n; k += nthreads()) sStatus[k] = 0;
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
                if (mh[c].y > 0 && !sensor) {
                    if (atomicMin(&sWake[bA], k) > k) sChanged = 1;
                    if (atomicMin(&sWake[bB], k) > k) sChanged = 1;
                }
                continue;
            }
            sStatus[k] = 1;
            if (update(c)) {
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
    if (tid() == 0) {
        int out = 0;
        for (int k = 0; k < n; ++k) {
            int c = order[k];
            if (sStatus[k] == 2) destroyContact(c);
            else order[out++] = c;
        }
        st->contactCount = out;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ contact solver
// b2ContactSolver (Dynamics/Contacts/b2ContactSolver.cpp) over one island's constraints.
struct Solver {
    VelConstraint* vc;
    PosConstraint* pc;
    int n;
    float4* pos;
    float4* vel;
};

__device__ inline Vec2 MulM(const float* A, Vec2 v) { return V(A[0] * v.x + A[2] * v.y, A[1] * v.x + A[3] * v.y); }

// b2ContactSolver::b2ContactSolver (b2ContactSolver.cpp:49-141). islandBase maps island-local body
// indices to rows of pos/vel.
__device__ void SolverSetup(Wd& W, Solver& S, const int* contacts, bool warmStarting, float dtRatio)
{
    for (int i = 0; i < S.n; ++i) {
        int c = contacts[i];
        int4 info = W.ci[c];
        int fA = info.y, fB = info.z;
        int bA = W.fixBody(fA), bB = W.fixBody(fB);
        float4 mA = W.mas[bA], mB = W.mas[bB];
        float4 pp = W.cp[c];
        int4 h = W.mh[c];
        float4 mvv = W.mv[c], p0 = W.mp0[c], p1 = W.mp1[c];
        VelConstraint& v = S.vc[i];
        PosConstraint& p = S.pc[i];
        v.friction = pp.x; v.restitution = pp.y; v.tangentSpeed = pp.z;
        // v.indexA / v.indexB were set when the island was built
        v.invMassA = mA.x; v.invMassB = mB.x; v.invIA = mA.y; v.invIB = mB.y;
        v.contact = c;
        v.pointCount = h.y;
        v.K[0] = v.K[1] = v.K[2] = v.K[3] = 0.0f;
        v.normalMass[0] = v.normalMass[1] = v.normalMass[2] = v.normalMass[3] = 0.0f;
        p.indexA = v.indexA; p.indexB = v.indexB;
        p.invMassA = mA.x; p.invMassB = mB.x;
        p.localCenterA = V(mA.z, mA.w); p.localCenterB = V(mB.z, mB.w);
        p.invIA = mA.y; p.invIB = mB.y;
        p.localNormal = V(mvv.x, mvv.y);
        p.localPoint = V(mvv.z, mvv.w);
        p.pointCount = h.y;
        p.radiusA = W.fm[fA].w; p.radiusB = W.fm[fB].w;
        p.type = h.x;
        for (int j = 0; j < h.y; ++j) {
            float4 q = j == 0 ? p0 : p1;
            VelPoint& vp = v.p[j];
            if (warmStarting) {
                vp.normalImpulse = dtRatio * q.z;
                vp.tangentImpulse = dtRatio * q.w;
            } else {
                vp.normalImpulse = 0.0f;
                vp.tangentImpulse = 0.0f;
            }
            vp.rA = V(0.0f, 0.0f); vp.rB = V(0.0f, 0.0f);
            vp.normalMass = 0.0f; vp.tangentMass = 0.0f; vp.velocityBias = 0.0f;
            p.localPoints[j] = V(q.x, q.y);
        }
    }
}

// b2ContactSolver::InitializeVelocityConstraints (b2ContactSolver.cpp:143-252)
__device__ void SolverInitVelocity(Wd& W, Solver& S)
{
    for (int i = 0; i < S.n; ++i) {
        VelConstraint& v = S.vc[i];
        const PosConstraint& p = S.pc[i];
        Manifold m;
        W.loadManifold(v.contact, m);
        float mA = v.invMassA, mB = v.invMassB, iA = v.invIA, iB = v.invIB;
        float4 pa = S.pos[v.indexA], pb = S.pos[v.indexB];
        float4 va = S.vel[v.indexA], vb = S.vel[v.indexB];
        Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
        Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
        float wA = va.z, wB = vb.z;
        Xf xfA, xfB;
        xfA.q = RotOf(pa.z);
        xfB.q = RotOf(pb.z);
        xfA.p = cA - Mul(xfA.q, p.localCenterA);
        xfB.p = cB - Mul(xfB.q, p.localCenterB);
        WorldManifold wm;
        WorldManifoldInit(&wm, m, xfA, p.radiusA, xfB, p.radiusB);
        v.normal = wm.normal;
        for (int j = 0; j < v.pointCount; ++j) {
            VelPoint& vp = v.p[j];
            vp.rA = wm.pts[j] - cA;
            vp.rB = wm.pts[j] - cB;
            float rnA = Cross(vp.rA, v.normal), rnB = Cross(vp.rB, v.normal);
            float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
            vp.normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
            Vec2 tangent = Cross(v.normal, 1.0f);
            float rtA = Cross(vp.rA, tangent), rtB = Cross(vp.rB, tangent);
            float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
            vp.tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
            vp.velocityBias = 0.0f;
            float vRel = Dot(v.normal, vB + Cross(wB, vp.rB) - vA - Cross(wA, vp.rA));
            if (vRel < -kVelocityThreshold) vp.velocityBias = -v.restitution * vRel;
        }
        if (v.pointCount == 2) {
            const VelPoint& p1 = v.p[0];
            const VelPoint& p2 = v.p[1];
            float rn1A = Cross(p1.rA, v.normal), rn1B = Cross(p1.rB, v.normal);
            float rn2A = Cross(p2.rA, v.normal), rn2B = Cross(p2.rB, v.normal);
            float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
            float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
            float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
            const float k_maxConditionNumber = 1000.0f;
            if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
                v.K[0] = k11; v.K[1] = k12; v.K[2] = k12; v.K[3] = k22;
                // b2Mat22::GetInverse (Common/b2Math.h:185-197)
                float a = v.K[0], b = v.K[2], cc = v.K[1], dd = v.K[3];
                float det = a * dd - b * cc;
                if (det != 0.0f) det = 1.0f / det;
                v.normalMass[0] = det * dd; v.normalMass[2] = -det * b;
                v.normalMass[1] = -det * cc; v.normalMass[3] = det * a;
            } else {
                v.pointCount = 1;
            }
        }
    }
}

// b2ContactSolver::WarmStart (b2ContactSolver.cpp:254-292)
__device__ void SolverWarmStart(Solver& S)
{
    for (int i = 0; i < S.n; ++i) {
        const VelConstraint& v = S.vc[i];
        float4 va = S.vel[v.indexA], vb = S.vel[v.indexB];
        Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
        float wA = va.z, wB = vb.z;
        Vec2 normal = v.normal, tangent = Cross(normal, 1.0f);
        for (int j = 0; j < v.pointCount; ++j) {
            const VelPoint& p = v.p[j];
            Vec2 P = p.normalImpulse * normal + p.tangentImpulse * tangent;
            wA -= v.invIA * Cross(p.rA, P);
            vA = vA - v.invMassA * P;
            wB += v.invIB * Cross(p.rB, P);
            vB = vB + v.invMassB * P;
        }
        S.vel[v.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
        S.vel[v.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
    }
}

// b2ContactSolver::SolveVelocityConstraints (b2ContactSolver.cpp:294-605): friction per point, then
// the normal constraint: one point, or the 2-point block LCP solved by total enumeration.
__device__ void SolverVelocity(Solver& S)
{
    for (int i = 0; i < S.n; ++i) {
        VelConstraint& v = S.vc[i];
        float mA = v.invMassA, iA = v.invIA, mB = v.invMassB, iB = v.invIB;
        float4 va = S.vel[v.indexA], vb = S.vel[v.indexB];
        Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
        float wA = va.z, wB = vb.z;
        Vec2 normal = v.normal, tangent = Cross(normal, 1.0f);
        float friction = v.friction;
        int pointCount = v.pointCount;
        for (int j = 0; j < pointCount; ++j) {
            VelPoint& p = v.p[j];
            Vec2 dv = vB + Cross(wB, p.rB) - vA - Cross(wA, p.rA);
            float vt = Dot(dv, tangent) - v.tangentSpeed;
            float lambda = p.tangentMass * (-vt);
            float maxFriction = friction * p.normalImpulse;
            float newImpulse = Clampf(p.tangentImpulse + lambda, -maxFriction, maxFriction);
            lambda = newImpulse - p.tangentImpulse;
            p.tangentImpulse = newImpulse;
            Vec2 P = lambda * tangent;
            vA = vA - mA * P;
            wA -= iA * Cross(p.rA, P);
            vB = vB + mB * P;
            wB += iB * Cross(p.rB, P);
        }
        if (pointCount == 1) {
            VelPoint& p = v.p[0];
            Vec2 dv = vB + Cross(wB, p.rB) - vA - Cross(wA, p.rA);
            float vn = Dot(dv, normal);
            float lambda = -p.normalMass * (vn - p.velocityBias);
            float newImpulse = Maxf(p.normalImpulse + lambda, 0.0f);
            lambda = newImpulse - p.normalImpulse;
            p.normalImpulse = newImpulse;
            Vec2 P = lambda * normal;
            vA = vA - mA * P;
            wA -= iA * Cross(p.rA, P);
            vB = vB + mB * P;
            wB += iB * Cross(p.rB, P);
        } else {
            VelPoint& cp1 = v.p[0];
            VelPoint& cp2 = v.p[1];
            Vec2 a = V(cp1.normalImpulse, cp2.normalImpulse);
            Vec2 dv1 = vB + Cross(wB, cp1.rB) - vA - Cross(wA, cp1.rA);
            Vec2 dv2 = vB + Cross(wB, cp2.rB) - vA - Cross(wA, cp2.rA);
            float vn1 = Dot(dv1, normal), vn2 = Dot(dv2, normal);
            Vec2 b;
            b.x = vn1 - cp1.velocityBias;
            b.y = vn2 - cp2.velocityBias;
            b = b - MulM(v.K, a);
            Vec2 x = -MulM(v.normalMass, b);
            bool solved = x.x >= 0.0f && x.y >= 0.0f;
            if (!solved) {
                x.x = -cp1.normalMass * b.x;
                x.y = 0.0f;
                vn2 = v.K[1] * x.x + b.y;
                solved = x.x >= 0.0f && vn2 >= 0.0f;
            }
            if (!solved) {
                x.x = 0.0f;
                x.y = -cp2.normalMass * b.y;
                vn1 = v.K[2] * x.y + b.x;
                solved = x.y >= 0.0f && vn1 >= 0.0f;
            }
            if (!solved) {
                x.x = 0.0f;
                x.y = 0.0f;
                vn1 = b.x;
                vn2 = b.y;
                solved = vn1 >= 0.0f && vn2 >= 0.0f;
            }
            if (solved) {
                Vec2 dd = x - a;
                Vec2 P1 = dd.x * normal, P2 = dd.y * normal;
                vA = vA - mA * (P1 + P2);
                wA -= iA * (Cross(cp1.rA, P1) + Cross(cp2.rA, P2));
                vB = vB + mB * (P1 + P2);
                wB += iB * (Cross(cp1.rB, P1) + Cross(cp2.rB, P2));
                cp1.normalImpulse = x.x;
                cp2.normalImpulse = x.y;
            }
        }
        S.vel[v.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
        S.vel[v.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
    }
}

// b2ContactSolver::StoreImpulses (b2ContactSolver.cpp:607-620)
__device__ void SolverStore(Wd& W, Solver& S)
{
    for (int i = 0; i < S.n; ++i) {
        const VelConstraint& v = S.vc[i];
        if (v.pointCount > 0) { W.mp0[v.contact].z = v.p[0].normalImpulse; W.mp0[v.contact].w = v.p[0].tangentImpulse; }
        if (v.pointCount > 1) { W.mp1[v.contact].z = v.p[1].normalImpulse; W.mp1[v.contact].w = v.p[1].tangentImpulse; }
    }
}

// b2ContactSolver::SolvePositionConstraints (b2ContactSolver.cpp:674-751) and
// SolveTOIPositionConstraints (:753-836) with b2PositionSolverManifold (:623-672).
__device__ bool SolverPosition(Solver& S, bool toi, int toiA, int toiB)
{
    float minSeparation = 0.0f;
    for (int i = 0; i < S.n; ++i) {
        const PosConstraint& p = S.pc[i];
        float mA, iA, mB, iB;
        if (!toi) { mA = p.invMassA; iA = p.invIA; mB = p.invMassB; iB = p.invIB; }
        else {
            mA = 0.0f; iA = 0.0f; mB = 0.0f; iB = 0.0f;
            if (p.indexA == toiA || p.indexA == toiB) { mA = p.invMassA; iA = p.invIA; }
            if (p.indexB == toiA || p.indexB == toiB) { mB = p.invMassB; iB = p.invIB; }
        }
        float4 pa = S.pos[p.indexA], pb = S.pos[p.indexB];
        Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
        float aA = pa.z, aB = pb.z;
        for (int j = 0; j < p.pointCount; ++j) {
            Xf xfA, xfB;
            xfA.q = RotOf(aA);
            xfB.q = RotOf(aB);
            xfA.p = cA - Mul(xfA.q, p.localCenterA);
            xfB.p = cB - Mul(xfB.q, p.localCenterB);
            Vec2 normal, point;
            float separation;
            if (p.type == kCircles) {
                Vec2 pA = Mul(xfA, p.localPoint), pB = Mul(xfB, p.localPoints[0]);
                normal = pB - pA;
                Normalize(normal);
                point = 0.5f * (pA + pB);
                separation = Dot(pB - pA, normal) - p.radiusA - p.radiusB;
            } else if (p.type == kFaceA) {
                normal = Mul(xfA.q, p.localNormal);
                Vec2 plane = Mul(xfA, p.localPoint);
                Vec2 clip = Mul(xfB, p.localPoints[j]);
                separation = Dot(clip - plane, normal) - p.radiusA - p.radiusB;
                point = clip;
            } else {
                normal = Mul(xfB.q, p.localNormal);
                Vec2 plane = Mul(xfB, p.localPoint);
                Vec2 clip = Mul(xfA, p.localPoints[j]);
                separation = Dot(clip - plane, normal) - p.radiusA - p.radiusB;
                point = clip;
                normal = -normal;
            }
            Vec2 rA = point - cA, rB = point - cB;
            minSeparation = Minf(minSeparation, separation);
            float C = toi ? Clampf(kToiBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f)
                          : Clampf(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
            float rnA = Cross(rA, normal), rnB = Cross(rB, normal);
            float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
            float impulse = K > 0.0f ? -C / K : 0.0f;
            Vec2 P = impulse * normal;
            cA = cA - mA * P;
            aA -= iA * Cross(rA, P);
            cB = cB + mB * P;
            aB += iB * Cross(rB, P);
        }
        S.pos[p.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
        S.pos[p.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    }
    return toi ? minSeparation >= -1.5f * kLinearSlop : minSeparation >= -3.0f * kLinearSlop;
}

// ------------------------------------------------------------------ revolute joint
// b2RevoluteJoint (Dynamics/Joints/b2RevoluteJoint.cpp:66-380); pos/vel rows are indexA/indexB,
// set when the island was built.
__device__ void RevInit(Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
{
    int A = j.bodyA, B = j.bodyB;
    float4 mA4 = W.mas[A], mB4 = W.mas[B];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    float aA = pos[j.indexA].z, aB = pos[j.indexB].z;
    float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
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
        if (Absf(j.upperAngle - j.lowerAngle) < 2.0f * kAngularSlop) j.limitState = 3;
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
    if (warmStarting) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        j.motorImpulse *= dtRatio;
        Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.motorImpulse + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.motorImpulse + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
        j.motorImpulse = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

// b2Mat33::Solve33 / Solve22 (Common/b2Math.cpp:24-56), columns ex = M[0..2], ey = M[3..5], ez = M[6..8]
__device__ inline void Solve33(const float* M, const float* b, float* x)
{
    float t[3];
    t[0] = M[4] * M[8] - M[5] * M[7]; t[1] = M[5] * M[6] - M[3] * M[8]; t[2] = M[3] * M[7] - M[4] * M[6];
    float det = M[0] * t[0] + M[1] * t[1] + M[2] * t[2];
    if (det != 0.0f) det = 1.0f / det;
    x[0] = det * (b[0] * t[0] + b[1] * t[1] + b[2] * t[2]);
    t[0] = b[1] * M[8] - b[2] * M[7]; t[1] = b[2] * M[6] - b[0] * M[8]; t[2] = b[0] * M[7] - b[1] * M[6];
    x[1] = det * (M[0] * t[0] + M[1] * t[1] + M[2] * t[2]);
    t[0] = M[4] * b[2] - M[5] * b[1]; t[1] = M[5] * b[0] - M[3] * b[2]; t[2] = M[3] * b[1] - M[4] * b[0];
    x[2] = det * (M[0] * t[0] + M[1] * t[1] + M[2] * t[2]);
}
__device__ inline Vec2 Solve22(const float* M, Vec2 b)
{
    float a11 = M[0], a12 = M[3], a21 = M[1], a22 = M[4];
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = 1.0f / det;
    return V(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}

__device__ void RevSolveVelocity(Joint& j, float4* vel, float dt)
{
    float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    bool fixedRotation = (iA + iB == 0.0f);
    if (j.enableMotor && j.limitState != 3 && !fixedRotation) {
        float Cdot = wB - wA - j.motorSpeed;
        float impulse = -j.motorMass * Cdot;
        float oldImpulse = j.motorImpulse;
        float maxImpulse = dt * j.maxMotorTorque;
        j.motorImpulse = Clampf(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if (j.enableLimit && j.limitState != 0 && !fixedRotation) {
        Vec2 Cdot1 = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        float Cdot2 = wB - wA;
        float Cd[3] = {Cdot1.x, Cdot1.y, Cdot2};
        float imp[3];
        Solve33(j.mass, Cd, imp);
        imp[0] = -imp[0]; imp[1] = -imp[1]; imp[2] = -imp[2];
        if (j.limitState == 3) {
            j.impulse[0] += imp[0]; j.impulse[1] += imp[1]; j.impulse[2] += imp[2];
        } else {
            float newImpulse = j.impulse[2] + imp[2];
            bool clampIt = j.limitState == 1 ? newImpulse < 0.0f : newImpulse > 0.0f;
            if (clampIt) {
                Vec2 rhs = -Cdot1 + j.impulse[2] * V(j.mass[6], j.mass[7]);
                Vec2 reduced = Solve22(j.mass, rhs);
                imp[0] = reduced.x; imp[1] = reduced.y; imp[2] = -j.impulse[2];
                j.impulse[0] += reduced.x; j.impulse[1] += reduced.y; j.impulse[2] = 0.0f;
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool RevSolvePosition(Joint& j, float4* pos)
{
    float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    float angularError = 0.0f, positionError = 0.0f;
    bool fixedRotation = (j.invIA + j.invIB == 0.0f);
    if (j.enableLimit && j.limitState != 0 && !fixedRotation) {
        float angle = aB - aA - j.referenceAngle;
        float limitImpulse = 0.0f;
        if (j.limitState == 3) {
            float C = Clampf(angle - j.lowerAngle, -kMaxAngularCorrection, kMaxAngularCorrection);
            limitImpulse = -j.motorMass * C;
            angularError = Absf(C);
        } else if (j.limitState == 1) {
            float C = angle - j.lowerAngle;
            angularError = -C;
            C = Clampf(C + kAngularSlop, -kMaxAngularCorrection, 0.0f);
            limitImpulse = -j.motorMass * C;
        } else if (j.limitState == 2) {
            float C = angle - j.upperAngle;
            angularError = C;
            C = Clampf(C - kAngularSlop, 0.0f, kMaxAngularCorrection);
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
        float K[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
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
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------------ island solve
// b2Island::Solve (Dynamics/b2Island.cpp:185-384) for island `island`, by one thread.
__device__ void Wd::islandSolve(int island, const StepParams& P, float h, float dtRatio)
{
    int4 isl = islands[island];
    int2 ij = islandJ[island];
    const int bBase = isl.x, nb = isl.y;
    const float gx = st->gx, gy = st->gy;
    for (int i = 0; i < nb; ++i) {
        int b = sBody[bBase + i];
        float4 s = sw[b];
        float4 v4 = vel[b];
        Vec2 v = V(v4.x, v4.y);
        float w = v4.z;
        sw0[b] = make_float4(s.x, s.y, s.z, sw0[b].w);
        if (type(b) == kDynamic) {
            float4 m = mas[b], pr = prop[b], f = frc[b];
            Vec2 g = pr.z * V(gx, gy);
            v = v + h * (g + m.x * V(f.x, f.y));
            w += h * m.y * f.z;
            v = (1.0f / (1.0f + h * pr.x)) * v;
            w *= 1.0f / (1.0f + h * pr.y);
        }
        sPos[bBase + i] = make_float4(s.x, s.y, s.z, 0.0f);
        sVel[bBase + i] = make_float4(v.x, v.y, w, 0.0f);
    }
    Solver S;
    S.vc = vc + isl.z;
    S.pc = pc + isl.z;
    S.n = isl.w;
    S.pos = sPos + bBase;
    S.vel = sVel + bBase;
    const bool warm = st->warmStarting != 0;
    SolverSetup(*this, S, sContact + isl.z, warm, dtRatio);
    SolverInitVelocity(*this, S);
    if (warm) SolverWarmStart(S);
    for (int k = 0; k < ij.y; ++k) RevInit(*this, jt[sJoint[ij.x + k]], S.pos, S.vel, warm, dtRatio);
    for (int it = 0; it < P.velocityIterations; ++it) {
        for (int k = 0; k < ij.y; ++k) RevSolveVelocity(jt[sJoint[ij.x + k]], S.vel, h);
        SolverVelocity(S);
    }
    SolverStore(*this, S);
    for (int i = 0; i < nb; ++i) {
        float4 p4 = S.pos[i], v4 = S.vel[i];
        Vec2 c = V(p4.x, p4.y), v = V(v4.x, v4.y);
        float a = p4.z, w = v4.z;
        Vec2 translation = h * v;
        if (Dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = kMaxTranslation / Length(translation);
            v.x *= ratio;
            v.y *= ratio;
        }
        float rotation = h * w;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = kMaxRotation / Absf(rotation);
            w *= ratio;
        }
        c = c + h * v;
        a += h * w;
        S.pos[i] = make_float4(c.x, c.y, a, 0.0f);
        S.vel[i] = make_float4(v.x, v.y, w, 0.0f);
    }
    bool positionSolved = false;
    for (int it = 0; it < P.positionIterations; ++it) {
        bool contactsOkay = SolverPosition(S, false, -1, -1);
        bool jointsOkay = true;
        for (int k = 0; k < ij.y; ++k) {
            bool ok = RevSolvePosition(jt[sJoint[ij.x + k]], S.pos);
            jointsOkay = jointsOkay && ok;
        }
        if (contactsOkay && jointsOkay) { positionSolved = true; break; }
    }
    // Write back (static bodies are shared between islands and never move: skipped).
    for (int i = 0; i < nb; ++i) {
        int b = sBody[bBase + i];
        if (type(b) == kStatic) continue;
        float4 p4 = S.pos[i], v4 = S.vel[i];
        sw[b] = make_float4(p4.x, p4.y, p4.z, sw[b].w);
        vel[b] = make_float4(v4.x, v4.y, v4.z, 0.0f);
        syncTransform(b);
    }
    int slept = 0;
    if (st->allowSleep) {
        float minSleepTime = kMaxFloat;
        const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
        const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
        for (int i = 0; i < nb; ++i) {
            int b = sBody[bBase + i];
            if (type(b) == kStatic) continue;
            float4 v4 = vel[b];
            float st0 = sw0[b].w;
            if ((flags(b) & kBAutoSleep) == 0 || v4.z * v4.z > angTolSqr || (v4.x * v4.x + v4.y * v4.y) > linTolSqr) {
                st0 = 0.0f;
                minSleepTime = 0.0f;
            } else {
                st0 += h;
                minSleepTime = Minf(minSleepTime, st0);
            }
            sw0[b].w = st0;
        }
        if (minSleepTime >= kTimeToSleep && positionSolved) {
            slept = 1;
            for (int i = 0; i < nb; ++i) {
                int b = sBody[bBase + i];
                if (type(b) != kStatic) setAwake(b, false);
            }
        }
    }
    sleepOut[island] = slept;
}

// ------------------------------------------------------------------ Solve
// b2World::Solve (Dynamics/b2World.cpp:388-577). The island DFS runs on one thread (it fixes the
// contact order inside every island); islands are then solved in parallel, one per thread, because
// they share no dynamic body.
__device__ void Wd::solve(const StepParams& P)
{
    __shared__ int sIslands;
    const int nb = d.bodyCount, nc = st->contactCount;
    for (int b = tid(); b < nb; b += nthreads()) bi[b].y &= ~kBIsland;
    for (int k = tid(); k < nc; k += nthreads()) ci[order[k]].x &= ~kCIsland;
    for (int j = tid(); j < d.jointCount; j += nthreads()) jt[j].islandFlag = 0;
    __syncthreads();
    if (tid() == 0) {
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
                vc[i].indexA = bj[fixBody(info.y)].z;
                vc[i].indexB = bj[fixBody(info.z)].z;
            }
            for (int i = jStart; i < jCur; ++i) {
                Joint& J = jt[sJoint[i]];
                J.indexA = bj[J.bodyA].z;
                J.indexB = bj[J.bodyB].z;
            }
            for (int i = bStart; i < bCur; ++i)
                if (bi[sBody[i]].x == kStatic) bi[sBody[i]].y &= ~kBIsland;
        }
        sIslands = nIsl;
        st->islands = nIsl;
        st->solvedBodies = movers;
        st->solvedContacts = cCur;
    }
    __syncthreads();
    const int nIsl = sIslands;
    const float dtRatio = st->inv_dt0 * P.dt;
    for (int i = tid(); i < nIsl; i += nthreads()) islandSolve(i, P, P.dt, dtRatio);
    __syncthreads();
    // A static body may sit in several islands; its awake flag ends as the last such island left it.
    if (tid() == 0) {
        for (int i = 0; i < nIsl; ++i) {
            int4 isl = islands[i];
            for (int k = isl.x; k < isl.x + isl.y; ++k) {
                int b = sBody[k];
                if (bi[b].x != kStatic) continue;
                if (sleepOut[i]) bi[b].y &= ~kBAwake;
                else bi[b].y |= kBAwake;
            }
        }
    }
    __syncthreads();
    for (int b = tid(); b < nb; b += nthreads()) {
        if ((bi[b].y & kBIsland) == 0 || bi[b].x == kStatic) continue;
        syncFixtures(b);
    }
    __syncthreads();
    findNewContacts();
}

// ------------------------------------------------------------------ SolveTOI
// b2World::SolveTOI (Dynamics/b2World.cpp:579-896). One event at a time, as the reference: thread 0
// scans the contact list in order (mutating sweeps as the reference does), the time of impact of every
// contact that needs one is computed in parallel, thread 0 takes the earliest, and sub-steps it.
__device__ void Wd::solveTOI(const StepParams& P)
{
    __shared__ int sN, sDone, sMin;
    __shared__ float sMinAlpha;
    if (st->stepComplete) {
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
    __syncthreads();
    for (int event = 0;; ++event) {
        // scan (sequential: body sweeps are advanced in list order)
        if (tid() == 0) {
            const int n = st->contactCount;
            for (int k = 0; k < n; ++k) {
                int c = order[k];
                TOITask& T = toi[k];
                T.contact = c;
                T.kind = 0;
                int4 info = ci[c];
                if ((info.x & kCEnabled) == 0) continue;
                if (info.w > kMaxSubSteps) continue;
                if (info.x & kCToi) { T.kind = 1; continue; }
                if (fi[info.y].w != 0 || fi[info.z].w != 0) continue;
                int bA = fixBody(info.y), bB = fixBody(info.z);
                int tA = bi[bA].x, tB = bi[bB].x;
                bool activeA = (bi[bA].y & kBAwake) && tA != kStatic;
                bool activeB = (bi[bB].y & kBAwake) && tB != kStatic;
                if (!activeA && !activeB) continue;
                bool collideA = (bi[bA].y & kBBullet) || tA != kDynamic;
                bool collideB = (bi[bB].y & kBBullet) || tB != kDynamic;
                if (!collideA && !collideB) continue;
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
                T.kind = 2;
                T.alpha0 = alpha0;
                T.sa = sA;
                T.sb = sB;
            }
            sN = n;
        }
        __syncthreads();
        const int n = sN;
        for (int k = tid(); k < n; k += nthreads()) {
            TOITask& T = toi[k];
            if (T.kind != 2) continue;
            int4 info = ci[T.contact];
            int state;
            float beta;
            TimeOfImpact(&state, &beta, ProxyOf(shape[info.y]), ProxyOf(shape[info.z]), T.sa, T.sb, 1.0f);
            float alpha = state == kToiTouching ? Minf(T.alpha0 + (1.0f - T.alpha0) * beta, 1.0f) : 1.0f;
            cp[T.contact].w = alpha;
            ci[T.contact].x = info.x | kCToi;
        }
        __syncthreads();
        if (tid() == 0) {
            int minC = kNullIdx;
            float minAlpha = 1.0f;
            for (int k = 0; k < n; ++k) {
                if (toi[k].kind == 0) continue;
                float alpha = cp[toi[k].contact].w;
                if (alpha < minAlpha) { minC = toi[k].contact; minAlpha = alpha; }
            }
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
        if (sDone) break;
        if (tid() == 0) {
            st->toiEvents = event + 1;
            const int mc = sMin;
            const float minAlpha = sMinAlpha;
            int4 info = ci[mc];
            int bA = fixBody(info.y), bB = fixBody(info.z);
            Sweep backup1 = sweep(bA), backup2 = sweep(bB);
            advance(bA, minAlpha);
            advance(bB, minAlpha);
            update(mc);
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
                        if (bi[other].x != kStatic) setAwake(other, true);
                        bj[other].z = nBodies;
                        sBody[nBodies++] = other;
                    }
                }
                // b2Island::SolveTOI (Dynamics/b2Island.cpp:386-485)
                float subDt = (1.0f - minAlpha) * P.dt;
                for (int i = 0; i < nBodies; ++i) {
                    int b = sBody[i];
                    float4 s = sw[b], v = vel[b];
                    sPos[i] = make_float4(s.x, s.y, s.z, 0.0f);
                    sVel[i] = make_float4(v.x, v.y, v.z, 0.0f);
                }
                Solver S;
                S.vc = vc; S.pc = pc; S.n = nContacts; S.pos = sPos; S.vel = sVel;
                for (int i = 0; i < nContacts; ++i) {
                    int4 ic = ci[sContact[i]];
                    vc[i].indexA = bj[fixBody(ic.y)].z;
                    vc[i].indexB = bj[fixBody(ic.z)].z;
                }
                SolverSetup(*this, S, sContact, false, 1.0f);
                const int toiA = bj[bA].z, toiB = bj[bB].z;
                for (int it = 0; it < 20; ++it)
                    if (SolverPosition(S, true, toiA, toiB)) break;
                {
                    float4 pA = sPos[toiA], pB = sPos[toiB];
                    float4 a0 = sw0[bA];
                    sw0[bA] = make_float4(pA.x, pA.y, pA.z, a0.w);
                    float4 b0 = sw0[bB];
                    sw0[bB] = make_float4(pB.x, pB.y, pB.z, b0.w);
                }
                SolverInitVelocity(*this, S);
                for (int it = 0; it < P.velocityIterations; ++it) SolverVelocity(S);
                float h = subDt;
                for (int i = 0; i < nBodies; ++i) {
                    float4 p4 = sPos[i], v4 = sVel[i];
                    Vec2 c = V(p4.x, p4.y), v = V(v4.x, v4.y);
                    float a = p4.z, w = v4.z;
                    Vec2 translation = h * v;
                    if (Dot(translation, translation) > kMaxTranslationSquared) {
                        float ratio = kMaxTranslation / Length(translation);
                        v.x *= ratio;
                        v.y *= ratio;
                    }
                    float rotation = h * w;
                    if (rotation * rotation > kMaxRotationSquared) {
                        float ratio = kMaxRotation / Absf(rotation);
                        w *= ratio;
                    }
                    c = c + h * v;
                    a += h * w;
                    sPos[i] = make_float4(c.x, c.y, a, 0.0f);
                    sVel[i] = make_float4(v.x, v.y, w, 0.0f);
                    int b = sBody[i];
                    sw[b] = make_float4(c.x, c.y, a, sw[b].w);
                    vel[b] = make_float4(v.x, v.y, w, 0.0f);
                    syncTransform(b);
                }
                for (int i = 0; i < nBodies; ++i) {
                    int b = sBody[i];
                    bi[b].y &= ~kBIsland;
                    if (bi[b].x != kDynamic) continue;
                    syncFixtures(b);
                    B2G_WALK(e, bi[b].w, eNext(e), 2 * d.contactCap + 2) ci[e >> 1].x &= ~(kCToi | kCIsland);
                }
            }
            sDone = skip ? 2 : 0;
        }
        __syncthreads();
        if (sDone == 2) continue;
        findNewContacts();
        if (st->subStepping) {
            if (tid() == 0) st->stepComplete = 0;
            __syncthreads();
            break;
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ kernels
// b2World::Step (Dynamics/b2World.cpp:899-963) for world schedule[blockIdx.x].
__global__ void __launch_bounds__(128) StepKernel(Batch B, StepParams P, const int* schedule)
{
    Wd W;
    W.init(B, schedule ? schedule[blockIdx.x] : blockIdx.x);
    const bool newFixture = W.st->newFixture != 0;
    __syncthreads();
    if (tid() == 0) {
        W.st->toiEvents = 0;
        W.st->islands = 0;
        W.st->solvedBodies = 0;
        W.st->solvedContacts = 0;
        W.st->pairsFound = 0;
        W.st->newFixture = 0;
    }
    __syncthreads();
    if (newFixture) W.findNewContacts();
    __syncthreads();
    W.collide();
    if (W.st->stepComplete && P.dt > 0.0f) W.solve(P);
    __syncthreads();
    if (W.st->continuous && P.dt > 0.0f) W.solveTOI(P);
    __syncthreads();
    for (int b = tid(); b < W.d.bodyCount; b += nthreads()) W.frc[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (tid() == 0 && P.dt > 0.0f) W.st->inv_dt0 = 1.0f / P.dt;
}

} // namespace b2g

// Launch entry used by the host runtime (b2g_api.cu).
cudaError_t b2gLaunchStep(const b2g::Batch& B, const b2g::StepParams& P, const int* schedule, int threads,
                          cudaStream_t stream)
{
    b2g::StepKernel<<<B.worlds, threads, 0, stream>>>(B, P, schedule);
    return cudaGetLastError();
}
