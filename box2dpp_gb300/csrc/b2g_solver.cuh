// Contact solver, revolute joint and island solve of the GB300 Box2D step (included by b2g_step.cu
// inside namespace b2g, after the world view Wd). Per-contact building blocks follow b2ContactSolver
// (Dynamics/Contacts/b2ContactSolver.cpp) and b2RevoluteJoint (Dynamics/Joints/b2RevoluteJoint.cpp)
// operation for operation. Island body rows (position, velocity) and the accumulated impulses are
// staged in shared memory when the world's islands fit; the read-only constraint records stay in
// global memory, are read with 128-bit loads, and the sequential sweeps prefetch the next record into
// L1 while solving the current one.
#pragma once

__device__ inline void PrefetchL1(const void* p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
template <typename T> __device__ inline void PrefetchRecord(const T* p)
{
    const char* c = reinterpret_cast<const char*>(p);
    for (int off = 0; off < (int)sizeof(T); off += 128) PrefetchL1(c + off);
}

// b2ContactSolver::b2ContactSolver, one contact (b2ContactSolver.cpp:61-139). v.idx.x / v.idx.y
// (body rows) are set when the island is built.
__device__ void ContactSetup(const Wd& W, VelConstraint& v, PosConstraint& p, float4& imp, int c, bool warmStarting,
                             float dtRatio)
{
    int4 info = W.ci[c];
    int fA = info.y, fB = info.z;
    int bA = W.fixBody(fA), bB = W.fixBody(fB);
    float4 mA = W.mas[bA], mB = W.mas[bB];
    float4 pp = W.cp[c];
    int4 h = W.mh[c];
    float4 mvv = W.mv[c], p0 = W.mp0[c], p1 = W.mp1[c];
    const int rowA = v.idx.x, rowB = v.idx.y;
    v.nf = make_float4(0.0f, 0.0f, pp.x, pp.z);
    v.m = make_float4(mA.x, mA.y, mB.x, mB.y);
    v.idx = make_int4(rowA, rowB, h.y, c);
    v.K = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v.NM = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v.r0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v.r1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    v.c0 = make_float4(0.0f, 0.0f, 0.0f, pp.y);
    v.c1 = make_float4(0.0f, 0.0f, 0.0f, pp.y);
    if (warmStarting) {
        imp = make_float4(dtRatio * p0.z, dtRatio * p0.w, h.y > 1 ? dtRatio * p1.z : 0.0f, h.y > 1 ? dtRatio * p1.w : 0.0f);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    p.lp = make_float4(p0.x, p0.y, h.y > 1 ? p1.x : 0.0f, h.y > 1 ? p1.y : 0.0f);
    p.ln = mvv;
    p.idx = make_int4(rowA, rowB, h.y, h.x);
    p.m = make_float4(mA.x, mA.y, mB.x, mB.y);
    p.lc = make_float4(mA.z, mA.w, mB.z, mB.w);
    p.rad = make_float4(W.fm[fA].w, W.fm[fB].w, 0.0f, 0.0f);
}

// b2ContactSolver::InitializeVelocityConstraints, one contact (b2ContactSolver.cpp:143-252)
__device__ void ContactInitVelocity(const Wd& W, VelConstraint& v, const PosConstraint& p, const float4* pos,
                                    const float4* vel, float2* sepOut = nullptr)
{
    Manifold m;
    W.loadManifold(v.idx.w, m);
    const float mA = v.m.x, iA = v.m.y, mB = v.m.z, iB = v.m.w;
    const float restitution = v.c0.w;
    float4 pa = pos[v.idx.x], pb = pos[v.idx.y];
    float4 va = vel[v.idx.x], vb = vel[v.idx.y];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    Xf xfA, xfB;
    xfA.q = RotOf(pa.z);
    xfB.q = RotOf(pb.z);
    xfA.p = cA - Mul(xfA.q, V(p.lc.x, p.lc.y));
    xfB.p = cB - Mul(xfB.q, V(p.lc.z, p.lc.w));
    WorldManifold wm;
    WorldManifoldInit(&wm, m, xfA, p.rad.x, xfB, p.rad.y);
    if (sepOut) *sepOut = make_float2(v.idx.z > 0 ? wm.sep[0] : 0.0f, v.idx.z > 1 ? wm.sep[1] : 0.0f);
    const Vec2 normal = wm.normal;
    v.nf.x = normal.x;
    v.nf.y = normal.y;
    const int pointCount = v.idx.z;
    Vec2 rA[2], rB[2];
    for (int j = 0; j < pointCount; ++j) {
        rA[j] = wm.pts[j] - cA;
        rB[j] = wm.pts[j] - cB;
        float rnA = Cross(rA[j], normal), rnB = Cross(rB[j], normal);
        float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        float normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
        Vec2 tangent = Cross(normal, 1.0f);
        float rtA = Cross(rA[j], tangent), rtB = Cross(rB[j], tangent);
        float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
        float tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
        float velocityBias = 0.0f;
        float vRel = Dot(normal, vB + Cross(wB, rB[j]) - vA - Cross(wA, rA[j]));
        if (vRel < -kVelocityThreshold) velocityBias = -restitution * vRel;
        float4 r4 = make_float4(rA[j].x, rA[j].y, rB[j].x, rB[j].y);
        float4 c4 = make_float4(normalMass, tangentMass, velocityBias, restitution);
        if (j == 0) { v.r0 = r4; v.c0 = c4; } else { v.r1 = r4; v.c1 = c4; }
    }
    if (pointCount == 2) {
        float rn1A = Cross(rA[0], normal), rn1B = Cross(rB[0], normal);
        float rn2A = Cross(rA[1], normal), rn2B = Cross(rB[1], normal);
        float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
        float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
        float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
        const float k_maxConditionNumber = 1000.0f;
        if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
            v.K = make_float4(k11, k12, k12, k22);
            // b2Mat22::GetInverse (Common/b2Math.h:185-197): a = ex.x, b = ey.x, c = ex.y, d = ey.y
            float a = k11, b = k12, cc = k12, dd = k22;
            float det = a * dd - b * cc;
            if (det != 0.0f) det = 1.0f / det;
            v.NM = make_float4(det * dd, -det * cc, -det * b, det * a);
        } else {
            v.idx.z = 1;
        }
    }
}

// b2ContactSolver::WarmStart, one contact (b2ContactSolver.cpp:254-292)
__device__ void ContactWarmStart(const VelConstraint& v, const float4 imp, float4* vel)
{
    float4 va = vel[v.idx.x], vb = vel[v.idx.y];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    Vec2 normal = V(v.nf.x, v.nf.y), tangent = Cross(normal, 1.0f);
    for (int j = 0; j < v.idx.z; ++j) {
        float4 r = j == 0 ? v.r0 : v.r1;
        float ni = j == 0 ? imp.x : imp.z, ti = j == 0 ? imp.y : imp.w;
        Vec2 P = ni * normal + ti * tangent;
        wA -= v.m.y * Cross(V(r.x, r.y), P);
        vA = vA - v.m.x * P;
        wB += v.m.w * Cross(V(r.z, r.w), P);
        vB = vB + v.m.z * P;
    }
    vel[v.idx.x] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[v.idx.y] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ inline Vec2 MulM4(float4 A, Vec2 v) { return V(A.x * v.x + A.z * v.y, A.y * v.x + A.w * v.y); }

// b2ContactSolver::SolveVelocityConstraints, one contact (b2ContactSolver.cpp:294-605): friction
// per point, then the normal constraint, one point or the 2-point block LCP by total enumeration.
__device__ __forceinline__ void ContactSolveVelocity(const VelConstraint& v, float4& imp, float4* vel)
{
    const float mA = v.m.x, iA = v.m.y, mB = v.m.z, iB = v.m.w;
    const int ia = v.idx.x, ib = v.idx.y, pointCount = v.idx.z;
    float4 va = vel[ia], vb = vel[ib];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Vec2 normal = V(v.nf.x, v.nf.y), tangent = Cross(normal, 1.0f);
    const float friction = v.nf.z, tangentSpeed = v.nf.w;
    const Vec2 rA0 = V(v.r0.x, v.r0.y), rB0 = V(v.r0.z, v.r0.w);
    const Vec2 rA1 = V(v.r1.x, v.r1.y), rB1 = V(v.r1.z, v.r1.w);
    float ni0 = imp.x, ti0 = imp.y, ni1 = imp.z, ti1 = imp.w;
    // friction, point 0 then point 1
    for (int j = 0; j < pointCount; ++j) {
        const Vec2 rA = j == 0 ? rA0 : rA1, rB = j == 0 ? rB0 : rB1;
        const float tangentMass = j == 0 ? v.c0.y : v.c1.y;
        const float normalImpulse = j == 0 ? ni0 : ni1;
        const float tangentImpulse = j == 0 ? ti0 : ti1;
        Vec2 dv = vB + Cross(wB, rB) - vA - Cross(wA, rA);
        float vt = Dot(dv, tangent) - tangentSpeed;
        float lambda = tangentMass * (-vt);
        float maxFriction = friction * normalImpulse;
        float newImpulse = Clampf(tangentImpulse + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - tangentImpulse;
        if (j == 0) ti0 = newImpulse; else ti1 = newImpulse;
        Vec2 P = lambda * tangent;
        vA = vA - mA * P;
        wA -= iA * Cross(rA, P);
        vB = vB + mB * P;
        wB += iB * Cross(rB, P);
    }
    if (pointCount == 1) {
        Vec2 dv = vB + Cross(wB, rB0) - vA - Cross(wA, rA0);
        float vn = Dot(dv, normal);
        float lambda = -v.c0.x * (vn - v.c0.z);
        float newImpulse = Maxf(ni0 + lambda, 0.0f);
        lambda = newImpulse - ni0;
        ni0 = newImpulse;
        Vec2 P = lambda * normal;
        vA = vA - mA * P;
        wA -= iA * Cross(rA0, P);
        vB = vB + mB * P;
        wB += iB * Cross(rB0, P);
    } else {
        Vec2 a = V(ni0, ni1);
        Vec2 dv1 = vB + Cross(wB, rB0) - vA - Cross(wA, rA0);
        Vec2 dv2 = vB + Cross(wB, rB1) - vA - Cross(wA, rA1);
        float vn1 = Dot(dv1, normal), vn2 = Dot(dv2, normal);
        Vec2 b;
        b.x = vn1 - v.c0.z;
        b.y = vn2 - v.c1.z;
        b = b - MulM4(v.K, a);
        Vec2 x = -MulM4(v.NM, b);
        bool solved = x.x >= 0.0f && x.y >= 0.0f;
        if (!solved) {
            x.x = -v.c0.x * b.x;
            x.y = 0.0f;
            vn2 = v.K.y * x.x + b.y;
            solved = x.x >= 0.0f && vn2 >= 0.0f;
        }
        if (!solved) {
            x.x = 0.0f;
            x.y = -v.c1.x * b.y;
            vn1 = v.K.z * x.y + b.x;
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
            wA -= iA * (Cross(rA0, P1) + Cross(rA1, P2));
            vB = vB + mB * (P1 + P2);
            wB += iB * (Cross(rB0, P1) + Cross(rB1, P2));
            ni0 = x.x;
            ni1 = x.y;
        }
    }
    imp = make_float4(ni0, ti0, ni1, ti1);
    vel[ia] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[ib] = make_float4(vB.x, vB.y, wB, 0.0f);
}

// b2ContactSolver::StoreImpulses, one contact (b2ContactSolver.cpp:607-620)
__device__ void ContactStore(Wd& W, const VelConstraint& v, const float4 imp)
{
    const int c = v.idx.w;
    if (v.idx.z > 0) { W.mp0[c].z = imp.x; W.mp0[c].w = imp.y; }
    if (v.idx.z > 1) { W.mp1[c].z = imp.z; W.mp1[c].w = imp.w; }
}

// b2ContactSolver::SolvePositionConstraints (b2ContactSolver.cpp:674-751) and
// SolveTOIPositionConstraints (:753-836) for one contact, with b2PositionSolverManifold (:623-672).
__device__ __forceinline__ void ContactSolvePosition(const PosConstraint& p, float4* pos, bool toi, int toiA, int toiB,
                                                     float& minSeparation)
{
    const int ia = p.idx.x, ib = p.idx.y, pointCount = p.idx.z, type = p.idx.w;
    float mA, iA, mB, iB;
    if (!toi) { mA = p.m.x; iA = p.m.y; mB = p.m.z; iB = p.m.w; }
    else {
        mA = 0.0f; iA = 0.0f; mB = 0.0f; iB = 0.0f;
        if (ia == toiA || ia == toiB) { mA = p.m.x; iA = p.m.y; }
        if (ib == toiA || ib == toiB) { mB = p.m.z; iB = p.m.w; }
    }
    const Vec2 localCenterA = V(p.lc.x, p.lc.y), localCenterB = V(p.lc.z, p.lc.w);
    const Vec2 localNormal = V(p.ln.x, p.ln.y), localPoint = V(p.ln.z, p.ln.w);
    const float radiusA = p.rad.x, radiusB = p.rad.y;
    float4 pa = pos[ia], pb = pos[ib];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    for (int j = 0; j < pointCount; ++j) {
        Xf xfA, xfB;
        xfA.q = RotOf(aA);
        xfB.q = RotOf(aB);
        xfA.p = cA - Mul(xfA.q, localCenterA);
        xfB.p = cB - Mul(xfB.q, localCenterB);
        const Vec2 lpj = j == 0 ? V(p.lp.x, p.lp.y) : V(p.lp.z, p.lp.w);
        Vec2 normal, point;
        float separation;
        if (type == kCircles) {
            Vec2 pA = Mul(xfA, localPoint), pB = Mul(xfB, V(p.lp.x, p.lp.y));
            normal = pB - pA;
            Normalize(normal);
            point = 0.5f * (pA + pB);
            separation = Dot(pB - pA, normal) - radiusA - radiusB;
        } else if (type == kFaceA) {
            normal = Mul(xfA.q, localNormal);
            Vec2 plane = Mul(xfA, localPoint);
            Vec2 clip = Mul(xfB, lpj);
            separation = Dot(clip - plane, normal) - radiusA - radiusB;
            point = clip;
        } else {
            normal = Mul(xfB.q, localNormal);
            Vec2 plane = Mul(xfB, localPoint);
            Vec2 clip = Mul(xfA, lpj);
            separation = Dot(clip - plane, normal) - radiusA - radiusB;
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
    pos[ia] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[ib] = make_float4(cB.x, cB.y, aB, 0.0f);
}

// Sequential sweeps over one island's constraints [lo, hi). The records are read-only during a sweep
// and their addresses are known ahead, so the records kSweepPrefetch places ahead are prefetched into
// L1 while the current one is solved (an L2 round trip is longer than one contact solve).
#ifndef B2G_SWEEP_PREFETCH
#define B2G_SWEEP_PREFETCH 4
#endif
constexpr int kSweepPrefetch = B2G_SWEEP_PREFETCH;
__device__ void SweepVelocity(const VelConstraint* vc, float4* imp, int lo, int hi, float4* vel)
{
    for (int i = lo; i < lo + kSweepPrefetch && i < hi; ++i) PrefetchRecord(vc + i);
    for (int i = lo; i < hi; ++i) {
        if (i + kSweepPrefetch < hi) PrefetchRecord(vc + i + kSweepPrefetch);
        const VelConstraint v = vc[i];
        float4 im = imp[i];
        ContactSolveVelocity(v, im, vel);
        imp[i] = im;
    }
}
__device__ bool SweepPosition(const PosConstraint* pc, int lo, int hi, float4* pos, bool toi, int toiA, int toiB,
                              float* minSepOut = nullptr)
{
    float minSeparation = 0.0f;
    for (int i = lo; i < lo + kSweepPrefetch && i < hi; ++i) PrefetchRecord(pc + i);
    for (int i = lo; i < hi; ++i) {
        if (i + kSweepPrefetch < hi) PrefetchRecord(pc + i + kSweepPrefetch);
        const PosConstraint p = pc[i];
        ContactSolvePosition(p, pos, toi, toiA, toiB, minSeparation);
    }
    if (minSepOut) *minSepOut = minSeparation;
    return toi ? minSeparation >= -1.5f * kLinearSlop : minSeparation >= -3.0f * kLinearSlop;
}

// ------------------------------------------------------------------ revolute joint
// b2RevoluteJoint (Dynamics/Joints/b2RevoluteJoint.cpp:66-380); pos/vel rows are indexA/indexB,
// set when the island is built.
__device__ void RevInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
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


// ------------------------------------------------------------------ distance joint
// b2DistanceJoint (Dynamics/Joints/b2DistanceJoint.cpp:61-225): a rod, or a spring when frequencyHz > 0.
__device__ void DistInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio, float dt)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    const Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    j.u = cB + j.rB - cA - j.rA;
    const float length = Length(j.u);
    if (length > kLinearSlop) {
        const float inv = 1.0f / length;
        j.u.x *= inv;
        j.u.y *= inv;
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
        const float h = dt;
        j.gamma = h * (d + h * k);
        j.gamma = j.gamma != 0.0f ? 1.0f / j.gamma : 0.0f;
        j.bias = C * h * k * j.gamma;
        invMass += j.gamma;
        j.motorMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
    } else {
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    if (warmStarting) {
        j.impulse[0] *= dtRatio;
        const Vec2 P = j.impulse[0] * j.u;
        vA = vA - j.invMassA * P;
        wA -= j.invIA * Cross(j.rA, P);
        vB = vB + j.invMassB * P;
        wB += j.invIB * Cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void DistSolveVelocity(Joint& j, float4* vel)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool DistSolvePosition(Joint& j, float4* pos)
{
    if (j.frequencyHz > 0.0f) return true;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    Vec2 u = cB + rB - cA - rA;
    const float length = Normalize(u);
    float C = length - j.length;
    C = Clampf(C, -kMaxLinearCorrection, kMaxLinearCorrection);
    const float impulse = -j.motorMass * C;
    const Vec2 P = impulse * u;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * Cross(rA, P);
    cB = cB + j.invMassB * P;
    aB += j.invIB * Cross(rB, P);
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return Absf(C) < kLinearSlop;
}

// ------------------------------------------------------------------ weld joint
// b2WeldJoint (Dynamics/Joints/b2WeldJoint.cpp:69-316); mass[] holds m_mass with columns ex = mass[0..2],
// ey = mass[3..5], ez = mass[6..8] (the Solve33 layout).
__device__ inline void WeldK(const Joint& j, Vec2 rA, Vec2 rB, float* K)
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
// b2Mat33::GetInverse22 and GetSymInverse33 (Common/b2Math.cpp:59-97)
__device__ inline void Inverse22(const float* K, float* M)
{
    const float a = K[0], b = K[3], c = K[1], d = K[4];
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    M[0] = det * d; M[3] = -det * b; M[2] = 0.0f;
    M[1] = -det * c; M[4] = det * a; M[5] = 0.0f;
    M[6] = 0.0f; M[7] = 0.0f; M[8] = 0.0f;
}
__device__ inline void SymInverse33(const float* K, float* M)
{
    // det = dot(ex, cross(ey, ez))
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

__device__ void WeldInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio, float dt)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float aA = pos[j.indexA].z, aB = pos[j.indexB].z;
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
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
        const float h = dt;
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
    if (warmStarting) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        const Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void WeldSolveVelocity(Joint& j, float4* vel)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float* M = j.mass;
    if (j.frequencyHz > 0.0f) {
        const float Cdot2 = wB - wA;
        const float impulse2 = -M[8] * (Cdot2 + j.bias + j.gamma * j.impulse[2]);
        j.impulse[2] += impulse2;
        wA -= iA * impulse2;
        wB += iB * impulse2;
        const Vec2 Cdot1 = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        // b2Mul22(m_mass, Cdot1)
        const Vec2 impulse1 = -V(M[0] * Cdot1.x + M[3] * Cdot1.y, M[1] * Cdot1.x + M[4] * Cdot1.y);
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
        // b2Mul(m_mass, Cdot) = Cdot.x * ex + Cdot.y * ey + Cdot.z * ez
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool WeldSolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
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
        angularError = Absf(C2);
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
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------------ prismatic joint
// b2PrismaticJoint (Dynamics/Joints/b2PrismaticJoint.cpp:128-487): body B slides along an axis fixed
// in body A, with a translation limit and a motor. lowerAngle/upperAngle hold the translation limits,
// maxMotorTorque the maximum motor force, u the axis of the step, mass[] the 3x3 K (Solve33 layout).
__device__ void PrisInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    const Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
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
    K[4] = iA + iB;
    if (K[4] == 0.0f) K[4] = 1.0f;  // fixed rotation
    K[5] = iA * j.a1 + iB * j.a2;
    K[8] = mA + mB + iA * j.a1 * j.a1 + iB * j.a2 * j.a2;
    K[3] = K[1]; K[6] = K[2]; K[7] = K[5];
    if (j.enableLimit) {
        const float translation = Dot(j.u, d);
        if (Absf(j.upperAngle - j.lowerAngle) < 2.0f * kLinearSlop) {
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
    if (warmStarting) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        j.motorImpulse *= dtRatio;
        const float axial = j.motorImpulse + j.impulse[2];
        const Vec2 P = j.impulse[0] * j.perp + axial * j.u;
        const float LA = j.impulse[0] * j.s1 + j.impulse[1] + axial * j.a1;
        const float LB = j.impulse[0] * j.s2 + j.impulse[1] + axial * j.a2;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
        j.motorImpulse = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void PrisSolveVelocity(Joint& j, float4* vel, float dt)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    if (j.enableMotor && j.limitState != 3) {
        const float Cdot = Dot(j.u, vB - vA) + j.a2 * wB - j.a1 * wA;
        float impulse = j.motorMass * (j.motorSpeed - Cdot);
        const float oldImpulse = j.motorImpulse;
        const float maxImpulse = dt * j.maxMotorTorque;
        j.motorImpulse = Clampf(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        const Vec2 P = impulse * j.u;
        const float LA = impulse * j.a1, LB = impulse * j.a2;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    const Vec2 Cdot1 = V(Dot(j.perp, vB - vA) + j.s2 * wB - j.s1 * wA, wB - wA);
    if (j.enableLimit && j.limitState != 0) {
        const float Cdot2 = Dot(j.u, vB - vA) + j.a2 * wB - j.a1 * wA;
        const float negCdot[3] = {-Cdot1.x, -Cdot1.y, -Cdot2};
        const float f1[3] = {j.impulse[0], j.impulse[1], j.impulse[2]};
        float df[3];
        Solve33(j.mass, negCdot, df);
        j.impulse[0] += df[0]; j.impulse[1] += df[1]; j.impulse[2] += df[2];
        if (j.limitState == 1) j.impulse[2] = Maxf(j.impulse[2], 0.0f);
        else if (j.limitState == 2) j.impulse[2] = Minf(j.impulse[2], 0.0f);
        // The 2x2 part re-solved with the clamped axial impulse (b2PrismaticJoint.cpp:322-327).
        const float dz = j.impulse[2] - f1[2];
        const Vec2 b = V(-Cdot1.x - dz * j.mass[6], -Cdot1.y - dz * j.mass[7]);
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
        const float LA = df.x * j.s1 + df.y, LB = df.x * j.s2 + df.y;
        vA = vA - mA * P;
        wA -= iA * LA;
        vB = vB + mB * P;
        wB += iB * LB;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool PrisSolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = cB + rB - cA - rA;
    const Vec2 axis = Mul(qA, j.localXAxisA);
    const float a1 = Cross(d + rA, axis), a2 = Cross(rB, axis);
    const Vec2 perp = Mul(qA, j.localYAxisA);
    const float s1 = Cross(d + rA, perp), s2 = Cross(rB, perp);
    const Vec2 C1 = V(Dot(perp, d), aB - aA - j.referenceAngle);
    float linearError = Absf(C1.x);
    const float angularError = Absf(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (j.enableLimit) {
        const float translation = Dot(axis, d);
        if (Absf(j.upperAngle - j.lowerAngle) < 2.0f * kLinearSlop) {
            C2 = Clampf(translation, -kMaxLinearCorrection, kMaxLinearCorrection);
            linearError = Maxf(linearError, Absf(translation));
            active = true;
        } else if (translation <= j.lowerAngle) {
            C2 = Clampf(translation - j.lowerAngle + kLinearSlop, -kMaxLinearCorrection, 0.0f);
            linearError = Maxf(linearError, j.lowerAngle - translation);
            active = true;
        } else if (translation >= j.upperAngle) {
            C2 = Clampf(translation - j.upperAngle - kLinearSlop, 0.0f, kMaxLinearCorrection);
            linearError = Maxf(linearError, translation - j.upperAngle);
            active = true;
        }
    }
    float imp[3];
    float K[9];
    K[0] = mA + mB + iA * s1 * s1 + iB * s2 * s2;
    K[1] = iA * s1 + iB * s2;
    K[4] = iA + iB;
    if (K[4] == 0.0f) K[4] = 1.0f;
    K[3] = K[1];
    if (active) {
        K[2] = iA * s1 * a1 + iB * s2 * a2;
        K[5] = iA * a1 + iB * a2;
        K[8] = mA + mB + iA * a1 * a1 + iB * a2 * a2;
        K[6] = K[2]; K[7] = K[5];
        const float negC[3] = {-C1.x, -C1.y, -C2};
        Solve33(K, negC, imp);
    } else {
        const Vec2 i1 = Solve22(K, -C1);
        imp[0] = i1.x; imp[1] = i1.y; imp[2] = 0.0f;
    }
    const Vec2 P = imp[0] * perp + imp[2] * axis;
    const float LA = imp[0] * s1 + imp[1] + imp[2] * a1;
    const float LB = imp[0] * s2 + imp[1] + imp[2] * a2;
    cA = cA - mA * P;
    aA -= iA * LA;
    cB = cB + mB * P;
    aB += iB * LB;
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return linearError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------------ wheel joint
// b2WheelJoint (Dynamics/Joints/b2WheelJoint.cpp:66-302): point-on-line with a spring along the axis
// and a rotational motor. The axis is taken as given (the reference's constructor does not normalise it).
__device__ void WheelInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio, float dt)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    const Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = cB + rB - cA - rA;
    j.ay = Mul(qA, j.localYAxisA);
    j.sAy = Cross(d + rA, j.ay);
    j.sBy = Cross(rB, j.ay);
    // the point-on-line mass (m_mass) is kept in mass[0]
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
            const float h = dt;
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
    if (warmStarting) {
        j.impulse[0] *= dtRatio;
        j.springImpulse *= dtRatio;
        j.motorImpulse *= dtRatio;
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void WheelSolveVelocity(Joint& j, float4* vel, float dt)
{
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    {   // spring
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
    {   // rotational motor
        const float Cdot = wB - wA - j.motorSpeed;
        float impulse = -j.motorMass * Cdot;
        const float oldImpulse = j.motorImpulse;
        const float maxImpulse = dt * j.maxMotorTorque;
        j.motorImpulse = Clampf(j.motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motorImpulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {   // point to line
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool WheelSolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    const Vec2 d = (cB - cA) + rB - rA;
    const Vec2 ay = Mul(qA, j.localYAxisA);
    const float sAy = Cross(d + rA, ay), sBy = Cross(rB, ay);
    const float C = Dot(d, ay);
    // the reference's mass here uses the lever arms of the velocity step (m_sAy, m_sBy)
    const float k = j.invMassA + j.invMassB + j.invIA * j.sAy * j.sAy + j.invIB * j.sBy * j.sBy;
    const float impulse = k != 0.0f ? -C / k : 0.0f;
    const Vec2 P = impulse * ay;
    const float LA = impulse * sAy, LB = impulse * sBy;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * LA;
    cB = cB + j.invMassB * P;
    aB += j.invIB * LB;
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return Absf(C) <= kLinearSlop;
}

// ------------------------------------------------------------------ rope joint
// b2RopeJoint (Dynamics/Joints/b2RopeJoint.cpp:45-198): a maximum distance between the anchors.
__device__ void RopeInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    const Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
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
    if (warmStarting) {
        j.impulse[0] *= dtRatio;
        const Vec2 P = j.impulse[0] * j.u;
        vA = vA - j.invMassA * P;
        wA -= j.invIA * Cross(j.rA, P);
        vB = vB + j.invMassB * P;
        wB += j.invIB * Cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void RopeSolveVelocity(Joint& j, float4* vel, float dt)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Vec2 vpA = vA + Cross(wA, j.rA);
    const Vec2 vpB = vB + Cross(wB, j.rB);
    const float C = j.ropeLength - j.maxLength;
    float Cdot = Dot(j.u, vpB - vpA);
    if (C < 0.0f) Cdot += (1.0f / dt) * C;  // predictive: the step's inv_dt
    float impulse = -j.motorMass * Cdot;
    const float oldImpulse = j.impulse[0];
    j.impulse[0] = Minf(0.0f, j.impulse[0] + impulse);
    impulse = j.impulse[0] - oldImpulse;
    const Vec2 P = impulse * j.u;
    vA = vA - j.invMassA * P;
    wA -= j.invIA * Cross(j.rA, P);
    vB = vB + j.invMassB * P;
    wB += j.invIB * Cross(j.rB, P);
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool RopeSolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    Vec2 u = cB + rB - cA - rA;
    const float length = Normalize(u);
    float C = length - j.maxLength;
    C = Clampf(C, 0.0f, kMaxLinearCorrection);
    const float impulse = -j.motorMass * C;
    const Vec2 P = impulse * u;
    cA = cA - j.invMassA * P;
    aA -= j.invIA * Cross(rA, P);
    cB = cB + j.invMassB * P;
    aB += j.invIB * Cross(rB, P);
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return length - j.maxLength < kLinearSlop;
}

// ------------------------------------------------------------------ friction and motor joints
// b2FrictionJoint (Dynamics/Joints/b2FrictionJoint.cpp:45-170): top-down friction, linear and angular
// impulses bounded by maxForce and maxTorque. b2MotorJoint (b2MotorJoint.cpp:58-200): drives body B
// to an offset from body A with bounded force and torque. Both have no position constraint.
// b2Mat22::GetInverse (Common/b2Math.h:245-257) of K (ex.x, ex.y, ey.x, ey.y in K[0..3]) into M.
__device__ inline void Mat22Inverse(const float* K, float* M)
{
    const float a = K[0], b = K[2], c = K[1], d = K[3];
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    M[0] = det * d; M[2] = -det * b;
    M[1] = -det * c; M[3] = det * a;
}

// the 2x2 linear mass and the angular mass of a friction or motor joint at this step's lever arms
__device__ inline void PointMasses(Joint& j)
{
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float K[4];
    K[0] = mA + mB + iA * j.rA.y * j.rA.y + iB * j.rB.y * j.rB.y;
    K[1] = -iA * j.rA.x * j.rA.y - iB * j.rB.x * j.rB.y;
    K[2] = K[1];
    K[3] = mA + mB + iA * j.rA.x * j.rA.x + iB * j.rB.x * j.rB.x;
    Mat22Inverse(K, j.mass);
    j.motorMass = iA + iB;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
}

__device__ void FrictionMotorInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
    if (j.type == kJointMotor) {
        j.rA = Mul(qA, -j.localCenterA);
        j.rB = Mul(qB, -j.localCenterB);
    } else {
        j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
        j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    }
    PointMasses(j);
    if (j.type == kJointMotor) {
        const Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
        j.linearError = cB + j.rB - cA - j.rA - Mul(qA, j.linearOffset);
        j.angularError = pb.z - pa.z - j.angularOffset;
    }
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    if (warmStarting) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio;
        j.impulse[2] *= dtRatio;
        const Vec2 P = V(j.impulse[0], j.impulse[1]);
        vA = vA - mA * P;
        wA -= iA * (Cross(j.rA, P) + j.impulse[2]);
        vB = vB + mB * P;
        wB += iB * (Cross(j.rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = 0.0f;
        j.impulse[2] = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void FrictionMotorSolveVelocity(Joint& j, float4* vel, float dt)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float h = dt;
    const bool motor = j.type == kJointMotor;
    const float invH = 1.0f / dt;
    {   // angular
        float Cdot = wB - wA;
        if (motor) Cdot = Cdot + invH * j.correctionFactor * j.angularError;
        float impulse = -j.motorMass * Cdot;
        const float oldImpulse = j.impulse[2];
        const float maxImpulse = h * j.maxTorque;
        j.impulse[2] = Clampf(j.impulse[2] + impulse, -maxImpulse, maxImpulse);
        impulse = j.impulse[2] - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {   // linear
        Vec2 Cdot = vB + Cross(wB, j.rB) - vA - Cross(wA, j.rA);
        if (motor) Cdot = Cdot + (invH * j.correctionFactor) * j.linearError;
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

// ------------------------------------------------------------------ mouse joint
// b2MouseJoint (Dynamics/Joints/b2MouseJoint.cpp:33-205): a soft spring pulling a point of body B to
// a target, force bounded by maxForce; body B's angular velocity is damped by 2% at each solve.
__device__ void MouseInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio, float dt)
{
    const float4 mB4 = W.mas[j.bodyB];
    j.localCenterB = V(mB4.z, mB4.w);
    j.invMassB = mB4.x; j.invIB = mB4.y;
    const float4 pb = pos[j.indexB], vb = vel[j.indexB];
    const Vec2 cB = V(pb.x, pb.y);
    Vec2 vB = V(vb.x, vb.y);
    float wB = vb.z;
    const Rot qB = RotOf(pb.z);
    const float mass = W.prop[j.bodyB].w;
    const float omega = 2.0f * kPi * j.frequencyHz;
    const float d = 2.0f * mass * j.dampingRatio * omega;
    const float k = mass * (omega * omega);
    const float h = dt;
    j.gamma = h * (d + h * k);
    if (j.gamma != 0.0f) j.gamma = 1.0f / j.gamma;
    j.beta = h * k * j.gamma;
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    float K[4];
    K[0] = j.invMassB + j.invIB * j.rB.y * j.rB.y + j.gamma;
    K[1] = -j.invIB * j.rB.x * j.rB.y;
    K[2] = K[1];
    K[3] = j.invMassB + j.invIB * j.rB.x * j.rB.x + j.gamma;
    Mat22Inverse(K, j.mass);
    j.mouseC = cB + j.rB - j.target;
    j.mouseC.x *= j.beta;
    j.mouseC.y *= j.beta;
    wB *= 0.98f;
    if (warmStarting) {
        j.impulse[0] *= dtRatio;
        j.impulse[1] *= dtRatio;
        const Vec2 I = V(j.impulse[0], j.impulse[1]);
        vB = vB + j.invMassB * I;
        wB += j.invIB * Cross(j.rB, I);
    } else {
        j.impulse[0] = j.impulse[1] = 0.0f;
    }
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void MouseSolveVelocity(Joint& j, float4* vel, float dt)
{
    const float4 vb = vel[j.indexB];
    Vec2 vB = V(vb.x, vb.y);
    float wB = vb.z;
    const Vec2 Cdot = vB + Cross(wB, j.rB);
    const Vec2 oldImpulse = V(j.impulse[0], j.impulse[1]);
    const Vec2 rhs = -(Cdot + j.mouseC + j.gamma * oldImpulse);
    const float* M = j.mass;
    Vec2 impulse = V(M[0] * rhs.x + M[2] * rhs.y, M[1] * rhs.x + M[3] * rhs.y);
    Vec2 total = oldImpulse + impulse;
    const float maxImpulse = dt * j.maxForce;
    if (LengthSq(total) > maxImpulse * maxImpulse) {
        const float s = maxImpulse / Length(total);
        total.x *= s;
        total.y *= s;
    }
    j.impulse[0] = total.x;
    j.impulse[1] = total.y;
    impulse = total - oldImpulse;
    vB = vB + j.invMassB * impulse;
    wB += j.invIB * Cross(j.rB, impulse);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

// ------------------------------------------------------------------ pulley joint
// b2PulleyJoint (Dynamics/Joints/b2PulleyJoint.cpp:53-275): lengthA + ratio * lengthB stays constant.
// The anchor-to-ground-anchor unit vectors of bodies A and B (zero when shorter than 10 linear slops).
__device__ inline void PulleyAxes(const Joint& j, Vec2 cA, Vec2 rA, Vec2 cB, Vec2 rB, Vec2& uA, Vec2& uB,
                                  float& lengthA, float& lengthB)
{
    uA = cA + rA - j.groundAnchorA;
    uB = cB + rB - j.groundAnchorB;
    lengthA = Length(uA);
    lengthB = Length(uB);
    if (lengthA > 10.0f * kLinearSlop) {
        const float inv = 1.0f / lengthA;
        uA.x *= inv;
        uA.y *= inv;
    } else {
        uA = V(0.0f, 0.0f);
    }
    if (lengthB > 10.0f * kLinearSlop) {
        const float inv = 1.0f / lengthB;
        uB.x *= inv;
        uB.y *= inv;
    } else {
        uB = V(0.0f, 0.0f);
    }
}

__device__ void PulleyInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invIA = mA4.y; j.invIB = mB4.y;
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = RotOf(pa.z), qB = RotOf(pb.z);
    j.rA = Mul(qA, j.localAnchorA - j.localCenterA);
    j.rB = Mul(qB, j.localAnchorB - j.localCenterB);
    float lengthA, lengthB;
    PulleyAxes(j, V(pa.x, pa.y), j.rA, V(pb.x, pb.y), j.rB, j.uA, j.uB, lengthA, lengthB);
    const float ruA = Cross(j.rA, j.uA), ruB = Cross(j.rB, j.uB);
    const float mA = j.invMassA + j.invIA * ruA * ruA;
    const float mB = j.invMassB + j.invIB * ruB * ruB;
    j.motorMass = mA + j.ratio * j.ratio * mB;
    if (j.motorMass > 0.0f) j.motorMass = 1.0f / j.motorMass;
    if (warmStarting) {
        j.impulse[0] *= dtRatio;
        const Vec2 PA = -(j.impulse[0]) * j.uA;
        const Vec2 PB = (-j.ratio * j.impulse[0]) * j.uB;
        vA = vA + j.invMassA * PA;
        wA += j.invIA * Cross(j.rA, PA);
        vB = vB + j.invMassB * PB;
        wB += j.invIB * Cross(j.rB, PB);
    } else {
        j.impulse[0] = 0.0f;
    }
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ void PulleySolveVelocity(Joint& j, float4* vel)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Vec2 vpA = vA + Cross(wA, j.rA);
    const Vec2 vpB = vB + Cross(wB, j.rB);
    const float Cdot = -Dot(j.uA, vpA) - j.ratio * Dot(j.uB, vpB);
    const float impulse = -j.motorMass * Cdot;
    j.impulse[0] += impulse;
    const Vec2 PA = -impulse * j.uA;
    const Vec2 PB = -j.ratio * impulse * j.uB;
    vA = vA + j.invMassA * PA;
    wA += j.invIA * Cross(j.rA, PA);
    vB = vB + j.invMassB * PB;
    wB += j.invIB * Cross(j.rB, PB);
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
}

__device__ bool PulleySolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB);
    const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
    const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
    Vec2 uA, uB;
    float lengthA, lengthB;
    PulleyAxes(j, cA, rA, cB, rB, uA, uB, lengthA, lengthB);
    const float ruA = Cross(rA, uA), ruB = Cross(rB, uB);
    const float mA = j.invMassA + j.invIA * ruA * ruA;
    const float mB = j.invMassB + j.invIB * ruB * ruB;
    float mass = mA + j.ratio * j.ratio * mB;
    if (mass > 0.0f) mass = 1.0f / mass;
    const float C = j.pulleyConstant - lengthA - j.ratio * lengthB;
    const float linearError = Absf(C);
    const float impulse = -mass * C;
    const Vec2 PA = -impulse * uA;
    const Vec2 PB = -j.ratio * impulse * uB;
    cA = cA + j.invMassA * PA;
    aA += j.invIA * Cross(rA, PA);
    cB = cB + j.invMassB * PB;
    aB += j.invIB * Cross(rB, PB);
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return linearError < kLinearSlop;
}

// ------------------------------------------------------------------ gear joint
// b2GearJoint (Dynamics/Joints/b2GearJoint.cpp:139-352): coordinate1 + ratio * coordinate2 stays
// constant, a coordinate being a revolute joint's relative angle or a prismatic joint's translation.
// Four bodies: A and B (the joints' bodies B) and C and D (their bodies A). The warm start does not
// scale the impulse by dtRatio, and the position solve always reports success.
__device__ void GearInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting)
{
    const float4 mA4 = W.mas[j.bodyA], mB4 = W.mas[j.bodyB], mC4 = W.mas[j.bodyC], mD4 = W.mas[j.bodyD];
    j.localCenterA = V(mA4.z, mA4.w); j.localCenterB = V(mB4.z, mB4.w);
    j.localCenterC = V(mC4.z, mC4.w); j.localCenterD = V(mD4.z, mD4.w);
    j.invMassA = mA4.x; j.invMassB = mB4.x; j.invMassC = mC4.x; j.invMassD = mD4.x;
    j.invIA = mA4.y; j.invIB = mB4.y; j.invIC = mC4.y; j.invID = mD4.y;
    const float4 va = vel[j.indexA], vb = vel[j.indexB], vc = vel[j.indexC], vd = vel[j.indexD];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y), vC = V(vc.x, vc.y), vD = V(vd.x, vd.y);
    float wA = va.z, wB = vb.z, wC = vc.z, wD = vd.z;
    const Rot qA = RotOf(pos[j.indexA].z), qB = RotOf(pos[j.indexB].z);
    const Rot qC = RotOf(pos[j.indexC].z), qD = RotOf(pos[j.indexD].z);
    float mass = 0.0f;
    if (j.gearTypeA == kJointRevolute) {
        j.JvAC = V(0.0f, 0.0f);
        j.JwA = 1.0f;
        j.JwC = 1.0f;
        mass += j.invIA + j.invIC;
    } else {
        const Vec2 u = Mul(qC, j.localAxisC);
        const Vec2 rC = Mul(qC, j.localAnchorC - j.localCenterC);
        const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
        j.JvAC = u;
        j.JwC = Cross(rC, u);
        j.JwA = Cross(rA, u);
        mass += j.invMassC + j.invMassA + j.invIC * j.JwC * j.JwC + j.invIA * j.JwA * j.JwA;
    }
    if (j.gearTypeB == kJointRevolute) {
        j.JvBD = V(0.0f, 0.0f);
        j.JwB = j.ratio;
        j.JwD = j.ratio;
        mass += j.ratio * j.ratio * (j.invIB + j.invID);
    } else {
        const Vec2 u = Mul(qD, j.localAxisD);
        const Vec2 rD = Mul(qD, j.localAnchorD - j.localCenterD);
        const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
        j.JvBD = j.ratio * u;
        j.JwD = j.ratio * Cross(rD, u);
        j.JwB = j.ratio * Cross(rB, u);
        mass += j.ratio * j.ratio * (j.invMassD + j.invMassB) + j.invID * j.JwD * j.JwD + j.invIB * j.JwB * j.JwB;
    }
    j.motorMass = mass > 0.0f ? 1.0f / mass : 0.0f;
    if (warmStarting) {
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
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
    vel[j.indexC] = make_float4(vC.x, vC.y, wC, 0.0f);
    vel[j.indexD] = make_float4(vD.x, vD.y, wD, 0.0f);
}

__device__ void GearSolveVelocity(Joint& j, float4* vel)
{
    const float4 va = vel[j.indexA], vb = vel[j.indexB], vc = vel[j.indexC], vd = vel[j.indexD];
    Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y), vC = V(vc.x, vc.y), vD = V(vd.x, vd.y);
    float wA = va.z, wB = vb.z, wC = vc.z, wD = vd.z;
    float Cdot = Dot(j.JvAC, vA - vC) + Dot(j.JvBD, vB - vD);
    Cdot += (j.JwA * wA - j.JwC * wC) + (j.JwB * wB - j.JwD * wD);
    const float impulse = -j.motorMass * Cdot;
    j.impulse[0] += impulse;
    vA = vA + (j.invMassA * impulse) * j.JvAC;
    wA += j.invIA * impulse * j.JwA;
    vB = vB + (j.invMassB * impulse) * j.JvBD;
    wB += j.invIB * impulse * j.JwB;
    vC = vC - (j.invMassC * impulse) * j.JvAC;
    wC -= j.invIC * impulse * j.JwC;
    vD = vD - (j.invMassD * impulse) * j.JvBD;
    wD -= j.invID * impulse * j.JwD;
    vel[j.indexA] = make_float4(vA.x, vA.y, wA, 0.0f);
    vel[j.indexB] = make_float4(vB.x, vB.y, wB, 0.0f);
    vel[j.indexC] = make_float4(vC.x, vC.y, wC, 0.0f);
    vel[j.indexD] = make_float4(vD.x, vD.y, wD, 0.0f);
}

__device__ bool GearSolvePosition(Joint& j, float4* pos)
{
    const float4 pa = pos[j.indexA], pb = pos[j.indexB], pc = pos[j.indexC], pd = pos[j.indexD];
    Vec2 cA = V(pa.x, pa.y), cB = V(pb.x, pb.y), cC = V(pc.x, pc.y), cD = V(pd.x, pd.y);
    float aA = pa.z, aB = pb.z, aC = pc.z, aD = pd.z;
    const Rot qA = RotOf(aA), qB = RotOf(aB), qC = RotOf(aC), qD = RotOf(aD);
    Vec2 JvAC, JvBD;
    float JwA, JwB, JwC, JwD, coordinateA, coordinateB;
    float mass = 0.0f;
    if (j.gearTypeA == kJointRevolute) {
        JvAC = V(0.0f, 0.0f);
        JwA = 1.0f;
        JwC = 1.0f;
        mass += j.invIA + j.invIC;
        coordinateA = aA - aC - j.referenceAngle;
    } else {
        const Vec2 u = Mul(qC, j.localAxisC);
        const Vec2 rC = Mul(qC, j.localAnchorC - j.localCenterC);
        const Vec2 rA = Mul(qA, j.localAnchorA - j.localCenterA);
        JvAC = u;
        JwC = Cross(rC, u);
        JwA = Cross(rA, u);
        mass += j.invMassC + j.invMassA + j.invIC * JwC * JwC + j.invIA * JwA * JwA;
        const Vec2 pC = j.localAnchorC - j.localCenterC;
        const Vec2 pA = MulT(qC, rA + (cA - cC));
        coordinateA = Dot(pA - pC, j.localAxisC);
    }
    if (j.gearTypeB == kJointRevolute) {
        JvBD = V(0.0f, 0.0f);
        JwB = j.ratio;
        JwD = j.ratio;
        mass += j.ratio * j.ratio * (j.invIB + j.invID);
        coordinateB = aB - aD - j.referenceAngleB;
    } else {
        const Vec2 u = Mul(qD, j.localAxisD);
        const Vec2 rD = Mul(qD, j.localAnchorD - j.localCenterD);
        const Vec2 rB = Mul(qB, j.localAnchorB - j.localCenterB);
        JvBD = j.ratio * u;
        JwD = j.ratio * Cross(rD, u);
        JwB = j.ratio * Cross(rB, u);
        mass += j.ratio * j.ratio * (j.invMassD + j.invMassB) + j.invID * JwD * JwD + j.invIB * JwB * JwB;
        const Vec2 pD = j.localAnchorD - j.localCenterD;
        const Vec2 pB = MulT(qD, rB + (cB - cD));
        coordinateB = Dot(pB - pD, j.localAxisD);
    }
    const float C = (coordinateA + j.ratio * coordinateB) - j.gearConstant;
    float impulse = 0.0f;
    if (mass > 0.0f) impulse = -C / mass;
    cA = cA + (j.invMassA * impulse) * JvAC;
    aA += j.invIA * impulse * JwA;
    cB = cB + (j.invMassB * impulse) * JvBD;
    aB += j.invIB * impulse * JwB;
    cC = cC - (j.invMassC * impulse) * JvAC;
    aC -= j.invIC * impulse * JwC;
    cD = cD - (j.invMassD * impulse) * JvBD;
    aD -= j.invID * impulse * JwD;
    pos[j.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    pos[j.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    pos[j.indexC] = make_float4(cC.x, cC.y, aC, 0.0f);
    pos[j.indexD] = make_float4(cD.x, cD.y, aD, 0.0f);
    return true;
}

// ------------------------------------------------------------------ joint dispatch
__device__ void JointInit(const Wd& W, Joint& j, float4* pos, float4* vel, bool warmStarting, float dtRatio, float dt)
{
    if (j.type == kJointWheel) WheelInit(W, j, pos, vel, warmStarting, dtRatio, dt);
    else if (j.type == kJointMouse) MouseInit(W, j, pos, vel, warmStarting, dtRatio, dt);
    else if (j.type == kJointPulley) PulleyInit(W, j, pos, vel, warmStarting, dtRatio);
    else if (j.type == kJointGear) GearInit(W, j, pos, vel, warmStarting);
    else if (j.type == kJointRope) RopeInit(W, j, pos, vel, warmStarting, dtRatio);
    else if (j.type == kJointFriction || j.type == kJointMotor) FrictionMotorInit(W, j, pos, vel, warmStarting, dtRatio);
    else if (j.type == kJointDistance) DistInit(W, j, pos, vel, warmStarting, dtRatio, dt);
    else if (j.type == kJointWeld) WeldInit(W, j, pos, vel, warmStarting, dtRatio, dt);
    else if (j.type == kJointPrismatic) PrisInit(W, j, pos, vel, warmStarting, dtRatio);
    else RevInit(W, j, pos, vel, warmStarting, dtRatio);
}
__device__ void JointSolveVelocity(Joint& j, float4* vel, float dt)
{
    if (j.type == kJointWheel) WheelSolveVelocity(j, vel, dt);
    else if (j.type == kJointMouse) MouseSolveVelocity(j, vel, dt);
    else if (j.type == kJointPulley) PulleySolveVelocity(j, vel);
    else if (j.type == kJointGear) GearSolveVelocity(j, vel);
    else if (j.type == kJointRope) RopeSolveVelocity(j, vel, dt);
    else if (j.type == kJointFriction || j.type == kJointMotor) FrictionMotorSolveVelocity(j, vel, dt);
    else if (j.type == kJointDistance) DistSolveVelocity(j, vel);
    else if (j.type == kJointWeld) WeldSolveVelocity(j, vel);
    else if (j.type == kJointPrismatic) PrisSolveVelocity(j, vel, dt);
    else RevSolveVelocity(j, vel, dt);
}
__device__ bool JointSolvePosition(Joint& j, float4* pos)
{
    if (j.type == kJointWheel) return WheelSolvePosition(j, pos);
    if (j.type == kJointMouse) return true;
    if (j.type == kJointPulley) return PulleySolvePosition(j, pos);
    if (j.type == kJointGear) return GearSolvePosition(j, pos);
    if (j.type == kJointRope) return RopeSolvePosition(j, pos);
    if (j.type == kJointFriction || j.type == kJointMotor) return true;
    if (j.type == kJointDistance) return DistSolvePosition(j, pos);
    if (j.type == kJointWeld) return WeldSolvePosition(j, pos);
    if (j.type == kJointPrismatic) return PrisSolvePosition(j, pos);
    return RevSolvePosition(j, pos);
}

// b2Island::Solve velocity/position integration clamps (Dynamics/b2Island.cpp:263-296, 442-470)
__device__ inline void IntegratePosition(float4& p4, float4& v4, float h)
{
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
    p4 = make_float4(c.x, c.y, a, 0.0f);
    v4 = make_float4(v.x, v.y, w, 0.0f);
}

// ------------------------------------------------------------------ residual
// Velocity residual of one contact (m/s): the natural-map residual of the contact's complementarity
// conditions in velocity units, i.e. for every point how far one projected Gauss-Seidel update of its
// impulse would move it, divided by the effective mass:
//   normal  |ni - max(0, ni - mn (vn - bias))| / mn  (= |vn - bias| for an active point that stays
//           active, = max(0, bias - vn) for an inactive one, = ni / mn for one that would separate)
//   tangent |ti - clamp(ti - mt vt, -mu ni, mu ni)| / mt  (= |vt| strictly inside the friction cone,
//           0 for a contact sliding at the bound in the direction its impulse opposes)
// It is zero exactly at a solution of the contact problem and does not change the solution.
__device__ float ContactResidual(const VelConstraint& v, const float4 imp, const float4* vel)
{
    const float4 va = vel[v.idx.x], vb = vel[v.idx.y];
    const Vec2 vA = V(va.x, va.y), vB = V(vb.x, vb.y);
    const Vec2 normal = V(v.nf.x, v.nf.y), tangent = Cross(normal, 1.0f);
    float r = 0.0f;
    for (int j = 0; j < v.idx.z; ++j) {
        const float4 rr = j == 0 ? v.r0 : v.r1;
        const float4 cc = j == 0 ? v.c0 : v.c1;
        const float ni = j == 0 ? imp.x : imp.z, ti = j == 0 ? imp.y : imp.w;
        const Vec2 dv = vB + Cross(vb.z, V(rr.z, rr.w)) - vA - Cross(va.z, V(rr.x, rr.y));
        const float vn = Dot(dv, normal);
        const float mn = cc.x, mt = cc.y;
        if (mn > 0.0f) r = fmaxf(r, fabsf(ni - fmaxf(0.0f, ni - mn * (vn - cc.z))) / mn);
        const float vt = Dot(dv, tangent) - v.nf.w;
        const float bound = v.nf.z * ni;
        if (mt > 0.0f) r = fmaxf(r, fabsf(ti - fminf(fmaxf(ti - mt * vt, -bound), bound)) / mt);
    }
    return r;
}

// CTA-wide maximum of non-negative floats (their bit patterns order as integers).
__device__ float ctaMaxNonNeg(float x, int* slot)
{
    __syncthreads();
    if (tid() == 0) *slot = 0;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    if ((tid() & 31) == 0 && x > 0.0f) atomicMax(slot, __float_as_int(x));
    __syncthreads();
    return __int_as_float(*slot);
}

// ------------------------------------------------------------------ learned warm start
// The 14 features of point j of a contact at the start of the velocity solve (after velocity
// integration, before any warm start): world normal (2), relative normal and tangent velocity of
// the point, its separation, the four inverse masses and inertias, the reference warm-start normal
// and tangent impulses (the previous step's, scaled by dtRatio; zero for new points) expressed as
// velocities (impulse / effective mass), the effective inverse normal mass, the friction
// coefficient, and whether the manifold has two points. The network predicts how far the point's
// final normal and tangent impulses are from the reference warm start, in the same velocity units.
__device__ void PointFeatures(const VelConstraint& v, const float4 imp, const float2 sep, const float4* vel, int j,
                              float (&f)[kMlpIn])
{
    const float4 va = vel[v.idx.x], vb = vel[v.idx.y];
    const float4 r = j == 0 ? v.r0 : v.r1;
    const float4 c = j == 0 ? v.c0 : v.c1;
    const Vec2 n = V(v.nf.x, v.nf.y), t = Cross(n, 1.0f);
    const Vec2 dv = V(vb.x, vb.y) + Cross(vb.z, V(r.z, r.w)) - V(va.x, va.y) - Cross(va.z, V(r.x, r.y));
    const float kn = c.x > 0.0f ? 1.0f / c.x : 0.0f, kt = c.y > 0.0f ? 1.0f / c.y : 0.0f;
    f[0] = n.x; f[1] = n.y;
    f[2] = Dot(dv, n);
    f[3] = Dot(dv, t) - v.nf.w;
    f[4] = j == 0 ? sep.x : sep.y;
    f[5] = v.m.x; f[6] = v.m.y; f[7] = v.m.z; f[8] = v.m.w;
    f[9] = (j == 0 ? imp.x : imp.z) * kn;
    f[10] = (j == 0 ? imp.y : imp.w) * kt;
    f[11] = kn;
    f[12] = v.nf.z;
    f[13] = v.idx.z == 2 ? 1.0f : 0.0f;
}

// Network predictions for every island contact point, written to vimpL: one 16-row tile (8
// contacts, 2 points each) per warp at a time; rows of absent points are zero and ignored. The
// outputs are corrections to the reference warm start in velocity units: normal impulse
// max(0, ref + y0 * normalMass), tangent impulse ref + y1 * tangentMass clamped to the friction
// cone (an output of zero reproduces the reference warm start). With kWarmLearned, points the
// reference starts warm (a positive normal impulse carried over) keep it: the network is used where
// the reference has nothing to offer, new or previously inactive points; kWarmLearnedAll corrects
// every point.
__device__ __noinline__ void Wd::learnedImpulses(const StepParams& P, int nContacts, const float4* imp, const float4* vel)
{
    // at most kLearnWarps warps evaluate tiles (their input tiles are static shared memory that every
    // launch of the kernel holds, so it is not sized for the widest CTA)
    constexpr int kLearnWarps = 8;
    __shared__ __align__(16) __nv_bfloat16 xTile[kLearnWarps][16 * kMlpInPad];
    const int warp = tid() >> 5, lane = tid() & 31, g = lane >> 2, t = lane & 3;
    const int warps = min(nthreads() >> 5, kLearnWarps);
    const int tiles = warp < warps ? (nContacts + 7) / 8 : 0;
    __nv_bfloat16* x = xTile[warp < warps ? warp : 0];
    for (int tile = warp; tile < tiles; tile += warps) {
        if (lane < 16) {
            const int i = 8 * tile + (lane >> 1), j = lane & 1;
            float f[kMlpIn];
            bool ok = false;
            if (i < nContacts) {
                const VelConstraint v = vc[i];
                if (j < v.idx.z) {
                    PointFeatures(v, imp[i], vsep[i], vel, j, f);
                    ok = true;
                }
            }
            for (int k = 0; k < kMlpInPad; ++k) {
                const float val = (ok && k < kMlpIn) ? (f[k] - P.mlp.mu[k]) / P.mlp.sigma[k] : 0.0f;
                x[lane * kMlpInPad + k] = __float2bfloat16_rn(val);
            }
        }
        __syncwarp();
        float out[4];
        MlpForwardTile(P.mlp, x, out);
        if (t == 0) {
            for (int h = 0; h < 2; ++h) {
                const int row = g + 8 * h, i = 8 * tile + (row >> 1), j = row & 1;
                if (i >= nContacts) continue;
                const VelConstraint v = vc[i];
                if (j >= v.idx.z) continue;
                const float4 c = j == 0 ? v.c0 : v.c1;
                const float4 ref = imp[i];
                const float niRef = j == 0 ? ref.x : ref.z, tiRef = j == 0 ? ref.y : ref.w;
                float ni = niRef, ti = tiRef;
                if (P.warmMode == kWarmLearnedAll || !(niRef > 0.0f)) {
                    ni = fmaxf(0.0f, niRef + out[2 * h] * c.x);
                    const float bound = v.nf.z * ni;
                    ti = fminf(fmaxf(tiRef + out[2 * h + 1] * c.y, -bound), bound);
                }
                float* dst = reinterpret_cast<float*>(&vimpL[i]) + 2 * j;
                dst[0] = ni;
                dst[1] = ti;
            }
        }
        __syncwarp();
    }
}

// Warm start of every island contact with impulses im on velocities v: per island in the reference
// order (plain), or colour by colour (coloured).
__device__ void Wd::warmStartAll(int nIsl, const int* colourStart, const float4* im, float4* v)
{
    if (colourStart == nullptr) {
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            const int4 I = islands[isl];
            for (int i = I.z; i < I.z + I.w; ++i) ContactWarmStart(vc[i], im[i], v);
        }
        __syncthreads();
        return;
    }
    for (int k = 0; k < kColours; ++k) {
        const int lo = colourStart[k], hi = colourStart[k + 1];
        if (lo == hi) continue;
        if (k == kSerialColour) {
            if (tid() == 0)
                for (int q = lo; q < hi; ++q) ContactWarmStart(vc[colourList[q]], im[colourList[q]], v);
        } else {
            for (int q = lo + tid(); q < hi; q += nthreads()) ContactWarmStart(vc[colourList[q]], im[colourList[q]], v);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ island solve
// b2Island::Solve (Dynamics/b2Island.cpp:185-384) for all islands of the world at once. Per-body and
// per-contact work that the reference does in independent loops (integration, constraint setup and
// initialisation, impulse storage, write-back) is spread over the CTA. The order-dependent work runs
// either per island on one thread in the reference's order (kSolverPlain), or colour by colour with
// the constraints of a colour spread over the CTA (kSolverColoured, colourStart != nullptr: contacts
// colourList[colourStart[k] .. colourStart[k+1]) have colour k; joints stay per island).
__device__ void Wd::solveIslands(const StepParams& P, int nIsl, int nRows, int nContacts, float4* smem, int smemRows,
                                 int smemContacts, const int* colourStart)
{
    __shared__ int sFlag, sRes;
    unsigned long long tStamp = clock64();
    const float h = P.dt;
    const float dtRatio = st->inv_dt0 * P.dt;
    const bool warm = st->warmStarting != 0;
    const float gx = st->gx, gy = st->gy;
    const bool rowsInSmem = nRows <= smemRows;
    const bool coloured = colourStart != nullptr;
    const bool learned = (P.warmMode == kWarmLearned || P.warmMode == kWarmLearnedAll) && warm;
    const bool logging = P.logX != nullptr && !coloured;
    const bool needSep = learned || logging;
    // island of each island contact during the learned warm-start choice (contact-sized scratch that
    // is free during the island solve)
    int* contactIsland = pairKeep;
    auto cColourIsland = [&](int i) -> int& { return contactIsland[i]; };
    float4* pos = rowsInSmem ? smem : sPos;
    float4* vel = rowsInSmem ? smem + smemRows : sVel;
    float4* imp = nContacts <= smemContacts ? smem + 2 * smemRows : vimp;
    // velocity integration (b2Island.cpp:190-222); c0 = c, a0 = a for every island body
    for (int r = tid(); r < nRows; r += nthreads()) {
        int b = sBody[r];
        float4 s = sw[b];
        float4 v4 = vel_body(b);
        Vec2 v = V(v4.x, v4.y);
        float w = v4.z;
        if (type(b) == kDynamic) {
            float4 m = mas[b], pr = prop[b], f = frc[b];
            Vec2 g = pr.z * V(gx, gy);
            v = v + h * (g + m.x * V(f.x, f.y));
            w += h * m.y * f.z;
            v = (1.0f / (1.0f + h * pr.x)) * v;
            w *= 1.0f / (1.0f + h * pr.y);
        }
        pos[r] = make_float4(s.x, s.y, s.z, 0.0f);
        vel[r] = make_float4(v.x, v.y, w, 0.0f);
        sw0[b] = make_float4(s.x, s.y, s.z, sw0[b].w);
    }
    __syncthreads();
    // constraint setup and initialisation, every island contact in parallel
    for (int i = tid(); i < nContacts; i += nthreads()) {
        VelConstraint v;
        v.idx = vc[i].idx;
        PosConstraint p;
        float4 im;
        ContactSetup(*this, v, p, im, sContact[i], warm, dtRatio);
        ContactInitVelocity(*this, v, p, pos, vel, needSep ? &vsep[i] : nullptr);
        vc[i] = v;
        pc[i] = p;
        imp[i] = im;
        if (logging) {
            // reserve the contact's log rows and write its features now (start of the solve)
            const int base = atomicAdd(P.logCount, v.idx.z);
            sStatus[i] = base;
            for (int j = 0; j < v.idx.z && base + j < P.logCap; ++j) {
                float f[kMlpIn];
                PointFeatures(v, im, vsep[i], vel, j, f);
                for (int k = 0; k < kMlpIn; ++k) P.logX[(size_t)(base + j) * kMlpIn + k] = f[k];
            }
        }
    }
    __syncthreads();
    // learned warm start: predictions, then both warm starts on their own velocity copies; the world
    // keeps the one whose velocity residual is smaller (the reference's on a tie)
    bool warmDone = false;
    if (learned && nContacts > 0) {
        learnedImpulses(P, nContacts, imp, vel);
        for (int r = tid(); r < nRows; r += nthreads()) sVelL[r] = vel[r];
        __syncthreads();
        warmStartAll(nIsl, colourStart, imp, vel);
        warmStartAll(nIsl, colourStart, vimpL, sVelL);
        // per-island residuals (islands are independent): each contact's residual both ways, reduced
        // into two per-island maxima (non-negative floats order as integers)
        int* islRef = sStack;
        int* islL = sWake;
        for (int isl = tid(); isl < nIsl; isl += nthreads()) { islRef[isl] = 0; islL[isl] = 0; }
        __syncthreads();
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            const int4 I = islands[isl];
            for (int i = I.z; i < I.z + I.w; ++i) cColourIsland(i) = isl;
        }
        __syncthreads();
        for (int i = tid(); i < nContacts; i += nthreads()) {
            const int isl = cColourIsland(i);
            atomicMax(&islRef[isl], __float_as_int(ContactResidual(vc[i], imp[i], vel)));
            atomicMax(&islL[isl], __float_as_int(ContactResidual(vc[i], vimpL[i], sVelL)));
        }
        __syncthreads();
        // each island keeps the warm start with the smaller residual (the reference's on a tie)
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            if (!(__int_as_float(islL[isl]) < __int_as_float(islRef[isl]))) continue;
            const int4 I = islands[isl];
            for (int r = I.x; r < I.x + I.y; ++r) vel[r] = sVelL[r];
            for (int i = I.z; i < I.z + I.w; ++i) imp[i] = vimpL[i];
            atomicAdd(&st->warmLearned, 1);
        }
        __syncthreads();
        float rRef = 0.0f, rL = 0.0f;
        (void)rRef;
        (void)rL;
        warmDone = true;
    }
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[8] = now - tStamp; tStamp = now; }
    int itersRun = P.velocityIterations;
    if (!coloured) {
        // order-dependent velocity phase per island, the reference's order
        if (tid() == 0) sFlag = 0;
        __syncthreads();
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            int4 I = islands[isl];
            int2 J = islandJ[isl];
            const int lo = I.z, hi = I.z + I.w;
            if (warm && !warmDone)
                for (int i = lo; i < hi; ++i) ContactWarmStart(vc[i], imp[i], vel);
            for (int k = 0; k < J.y; ++k) JointInit(*this, jt[sJoint[J.x + k]], pos, vel, warm, dtRatio, h);
            int it = 0;
            for (; it < P.velocityIterations; ++it) {
                if (P.tolerance > 0.0f) {
                    float r = 0.0f;
                    for (int i = lo; i < hi; ++i) r = fmaxf(r, ContactResidual(vc[i], imp[i], vel));
                    if (r <= P.tolerance) break;
                }
                for (int k = 0; k < J.y; ++k) JointSolveVelocity(jt[sJoint[J.x + k]], vel, h);
                SweepVelocity(vc, imp, lo, hi, vel);
            }
            atomicMax(&sFlag, it);
            atomicAdd(&st->velItersSum, it * I.w);
        }
        __syncthreads();
        itersRun = sFlag;
    } else {
        // colour by colour: warm start, joint initialisation per island, then the iterations
        const int nCol = kColours;
        if (warm && !warmDone) {
            for (int k = 0; k < nCol; ++k) {
                const int lo = colourStart[k], hi = colourStart[k + 1];
                if (lo == hi) continue;
                if (k == kSerialColour) {
                    if (tid() == 0)
                        for (int q = lo; q < hi; ++q) ContactWarmStart(vc[colourList[q]], imp[colourList[q]], vel);
                } else {
                    for (int q = lo + tid(); q < hi; q += nthreads()) ContactWarmStart(vc[colourList[q]], imp[colourList[q]], vel);
                }
                __syncthreads();
            }
        }
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            int2 J = islandJ[isl];
            for (int k = 0; k < J.y; ++k) JointInit(*this, jt[sJoint[J.x + k]], pos, vel, warm, dtRatio, h);
        }
        __syncthreads();
        int it = 0;
        for (; it < P.velocityIterations; ++it) {
            if (P.tolerance > 0.0f) {
                float r = 0.0f;
                for (int i = tid(); i < nContacts; i += nthreads()) r = fmaxf(r, ContactResidual(vc[i], imp[i], vel));
                if (ctaMaxNonNeg(r, &sRes) <= P.tolerance) break;
            }
            if (d.jointCount > 0) {
                for (int isl = tid(); isl < nIsl; isl += nthreads()) {
                    int2 J = islandJ[isl];
                    for (int k = 0; k < J.y; ++k) JointSolveVelocity(jt[sJoint[J.x + k]], vel, h);
                }
                __syncthreads();
            }
            for (int k = 0; k < nCol; ++k) {
                const int lo = colourStart[k], hi = colourStart[k + 1];
                if (lo == hi) continue;
                if (k == kSerialColour) {
                    if (tid() == 0)
                        for (int q = lo; q < hi; ++q) {
                            const int i = colourList[q];
                            float4 im = imp[i];
                            ContactSolveVelocity(vc[i], im, vel);
                            imp[i] = im;
                        }
                } else {
                    for (int q = lo + tid(); q < hi; q += nthreads()) {
                        const int i = colourList[q];
                        const VelConstraint v = vc[i];
                        float4 im = imp[i];
                        ContactSolveVelocity(v, im, vel);
                        imp[i] = im;
                    }
                }
                __syncthreads();
            }
        }
        itersRun = it;
        if (tid() == 0) st->velItersSum = it * nContacts;
    }
    if (P.measureResidual) {
        float r = 0.0f;
        for (int i = tid(); i < nContacts; i += nthreads()) r = fmaxf(r, ContactResidual(vc[i], imp[i], vel));
        r = ctaMaxNonNeg(r, &sRes);
        if (tid() == 0) st->residual = r;
    }
    if (tid() == 0) st->velIters = itersRun;
    if (logging) {
        for (int i = tid(); i < nContacts; i += nthreads()) {
            const VelConstraint v = vc[i];
            const float4 im = imp[i];
            const int base = sStatus[i];
            for (int j = 0; j < v.idx.z && base + j < P.logCap; ++j) {
                const float4 c = j == 0 ? v.c0 : v.c1;
                const float kn = c.x > 0.0f ? 1.0f / c.x : 0.0f, kt = c.y > 0.0f ? 1.0f / c.y : 0.0f;
                P.logT[2 * (size_t)(base + j)] = (j == 0 ? im.x : im.z) * kn;
                P.logT[2 * (size_t)(base + j) + 1] = (j == 0 ? im.y : im.w) * kt;
            }
        }
    }
    __syncthreads();
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[9] = now - tStamp; tStamp = now; }
    // impulses back to the manifolds, positions integrated, both in parallel
    for (int i = tid(); i < nContacts; i += nthreads()) ContactStore(*this, vc[i], imp[i]);
    for (int r = tid(); r < nRows; r += nthreads()) {
        float4 p4 = pos[r], v4 = vel[r];
        IntegratePosition(p4, v4, h);
        pos[r] = p4;
        vel[r] = v4;
    }
    __syncthreads();
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[10] = now - tStamp; tStamp = now; }
    if (!coloured) {
        // order-dependent position phase per island
        for (int isl = tid(); isl < nIsl; isl += nthreads()) {
            int4 I = islands[isl];
            int2 J = islandJ[isl];
            bool positionSolved = false;
            for (int it = 0; it < P.positionIterations; ++it) {
                float minSep = 0.0f;
                bool contactsOkay = SweepPosition(pc, I.z, I.z + I.w, pos, false, -1, -1, &minSep);
                if (it == 0 && minSep < 0.0f) atomicMax(reinterpret_cast<int*>(&st->maxPenetration), __float_as_int(-minSep));
                bool jointsOkay = true;
                for (int k = 0; k < J.y; ++k) {
                    bool ok = JointSolvePosition(jt[sJoint[J.x + k]], pos);
                    jointsOkay = jointsOkay && ok;
                }
                if (contactsOkay && jointsOkay) { positionSolved = true; break; }
            }
            sleepOut[isl] = positionSolved ? 1 : 0;
        }
    } else {
        // colour by colour; the early exit is taken for the whole world at once
        bool positionSolved = false;
        for (int it = 0; it < P.positionIterations; ++it) {
            float minSep = 0.0f;
            for (int k = 0; k < kColours; ++k) {
                const int lo = colourStart[k], hi = colourStart[k + 1];
                if (lo == hi) continue;
                if (k == kSerialColour) {
                    if (tid() == 0)
                        for (int q = lo; q < hi; ++q) ContactSolvePosition(pc[colourList[q]], pos, false, -1, -1, minSep);
                } else {
                    for (int q = lo + tid(); q < hi; q += nthreads()) {
                        const PosConstraint p = pc[colourList[q]];
                        ContactSolvePosition(p, pos, false, -1, -1, minSep);
                    }
                }
                __syncthreads();
            }
            bool jointsOkay = true;
            if (d.jointCount > 0) {
                for (int isl = tid(); isl < nIsl; isl += nthreads()) {
                    int2 J = islandJ[isl];
                    for (int k = 0; k < J.y; ++k) {
                        bool ok = JointSolvePosition(jt[sJoint[J.x + k]], pos);
                        jointsOkay = jointsOkay && ok;
                    }
                }
            }
            // every thread reports its worst separation (as a violation >= 0) and joint state
            const float violation = fmaxf(0.0f, -minSep);
            if (it == 0 && violation > 0.0f) atomicMax(reinterpret_cast<int*>(&st->maxPenetration), __float_as_int(violation));
            const float worst = ctaMaxNonNeg(jointsOkay ? violation : 1e30f, &sRes);
            if (worst <= 3.0f * kLinearSlop) { positionSolved = true; break; }
        }
        for (int isl = tid(); isl < nIsl; isl += nthreads()) sleepOut[isl] = positionSolved ? 1 : 0;
    }
    __syncthreads();
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[11] = now - tStamp; tStamp = now; }
    // write back and SynchronizeTransform (static bodies never move: skipped)
    for (int r = tid(); r < nRows; r += nthreads()) {
        int b = sBody[r];
        if (type(b) == kStatic) continue;
        float4 p4 = pos[r], v4 = vel[r];
        sw[b] = make_float4(p4.x, p4.y, p4.z, sw[b].w);
        vel_body(b) = make_float4(v4.x, v4.y, v4.z, 0.0f);
        syncTransform(b);
    }
    // b2Island::Report (b2Island.cpp:344, 518-541): PostSolve for every island contact, islands in
    // order, with the impulses the velocity iterations ended with
    if (evLog) {
        const int base = st->eventCount;
        __syncthreads();
        for (int i = tid(); i < nContacts; i += nthreads()) {
            const int4 info = ci[sContact[i]];
            const float4 im = imp[i];
            const int n = vc[i].idx.z;
            putEvent(base + i, kEvPostSolve, info.y, info.z, n, n > 0 ? im.x : 0.0f, n > 1 ? im.z : 0.0f,
                     n > 0 ? im.y : 0.0f, n > 1 ? im.w : 0.0f);
        }
        __syncthreads();
        if (tid() == 0) st->eventCount = base + nContacts;
    }
    __syncthreads();
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[12] = now - tStamp; tStamp = now; }
    // sleep (b2Island.cpp:346-383), per island
    for (int isl = tid(); isl < nIsl; isl += nthreads()) {
        int slept = 0;
        if (st->allowSleep) {
            int4 I = islands[isl];
            const bool positionSolved = sleepOut[isl] != 0;
            float minSleepTime = kMaxFloat;
            const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
            const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
            for (int r = I.x; r < I.x + I.y; ++r) {
                int b = sBody[r];
                if (type(b) == kStatic) continue;
                float4 v4 = vel_body(b);
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
                for (int r = I.x; r < I.x + I.y; ++r) {
                    int b = sBody[r];
                    if (type(b) != kStatic) setAwake(b, false);
                }
            }
        }
        sleepOut[isl] = slept;
    }
    __syncthreads();
    if (tid() == 0) { unsigned long long now = clock64(); st->cyc[13] = now - tStamp; tStamp = now; }
}
