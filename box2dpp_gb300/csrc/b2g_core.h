// Box2D per-step arithmetic for GB300: vector/rotation math, the project sin/cos, shape setup,
// narrowphase manifolds, GJK distance and time of impact. Compiled for the device (kernels) and the
// host (shape setup at body/fixture creation) with fused multiply-add disabled, so every float
// operation rounds exactly where the reference Box2D 2.3.2 rounds it (x86-64 SSE, no FMA).
//
// Reference citations are paths under Regression/box2d-ref/Box2DRef/ of the reference tree.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector_types.h>

#include "b2g_trig_table.h"

#ifdef __CUDACC__
#define B2G_HD __host__ __device__ __forceinline__
#define B2G_HDNI static __host__ __device__ __noinline__
#else
#define B2G_HD inline
#define B2G_HDNI static inline
#endif

namespace b2g {

// ------------------------------------------------------------------ settings (Common/b2Settings.h:44-160)
constexpr float kEpsilon = FLT_EPSILON;
constexpr float kMaxFloat = FLT_MAX;
constexpr float kPi = 3.14159265359f;
constexpr int kMaxPolyVerts = 8;
constexpr float kAabbExtension = 0.1f;
constexpr float kAabbMultiplier = 2.0f;
constexpr float kLinearSlop = 0.005f;
constexpr float kAngularSlop = 2.0f / 180.0f * kPi;
constexpr float kPolygonRadius = 2.0f * kLinearSlop;
constexpr int kMaxSubSteps = 8;
constexpr int kMaxTOIContacts = 32;
constexpr float kVelocityThreshold = 1.0f;
constexpr float kMaxLinearCorrection = 0.2f;
constexpr float kMaxAngularCorrection = 8.0f / 180.0f * kPi;
constexpr float kMaxTranslation = 2.0f;
constexpr float kMaxTranslationSquared = kMaxTranslation * kMaxTranslation;
constexpr float kMaxRotation = 0.5f * kPi;
constexpr float kMaxRotationSquared = kMaxRotation * kMaxRotation;
constexpr float kBaumgarte = 0.2f;
constexpr float kToiBaumgarte = 0.75f;
constexpr float kTimeToSleep = 0.5f;
constexpr float kLinearSleepTolerance = 0.01f;
constexpr float kAngularSleepTolerance = 2.0f / 180.0f * kPi;

// ------------------------------------------------------------------ project sin/cos
// One deterministic float sin/cos evaluated identically on every device and host, in float
// arithmetic only (GB300's FP64 is far slower than FP32):
//   1. k = rint(x * 256/pi); r = x - k*pi/256 as a float-float pair (rh, rl): pi/256 = C1 + C2 + C3,
//      the products k*C1 and k*C2 made exact with fused multiply-adds, the differences with TwoSum.
//   2. sin r = r + r^3(-1/6 + r^2/120) and cos r = 1 - r^2/2 + r^4/24 as float-float pairs
//      (|r| <= pi/512, so the corrections are ~1e-6 relative and float precision suffices for them).
//   3. sin x = S_j cos r + C_j sin r, cos x = C_j cos r - S_j sin r with float-float table values at
//      j = k mod 512, exact products by fused multiply-add, one final rounding to float.
// Within ~2^-41 of the exact value before the last rounding: the correctly rounded float except for
// about one input in 10^5. The only fused operations are the explicit fmaf calls (the build disables
// contraction everywhere else), so host and device round identically.
#ifdef __CUDACC__
static __device__ const __align__(16) float kTrigTableDev[512 * 4] = {B2G_TRIG_TABLE_ROWS};
#endif
static const float kTrigTableHost[512 * 4] = {B2G_TRIG_TABLE_ROWS};

B2G_HD const float* TrigTable()
{
#ifdef __CUDA_ARCH__
    return kTrigTableDev;
#else
    return kTrigTableHost;
#endif
}

B2G_HD void SinCos(float x, float* s_out, float* c_out)
{
    if (x == 0.0f) { *s_out = x; *c_out = 1.0f; return; }
    if (!(fabsf(x) <= FLT_MAX)) { *s_out = x - x; *c_out = x - x; return; }
    const float kf = rintf(x * B2G_INV_PIO256);
    const int idx = fabsf(kf) < 16777216.0f ? ((int)kf) & 511 : ((int)fmodf(kf, 512.0f)) & 511;
    // r = x - k*pi/256 in float-float
    const float p = kf * B2G_PIO256_1;
    const float pe = fmaf(kf, B2G_PIO256_1, -p);
    const float t = x - p;
    const float q = kf * B2G_PIO256_2;
    const float qe = fmaf(kf, B2G_PIO256_2, -q);
    const float s1 = t - pe;
    const float b1 = s1 - t;
    const float s1e = (t - (s1 - b1)) + (-pe - b1);
    const float s2 = s1 - q;
    const float b2 = s2 - s1;
    const float s2e = (s1 - (s2 - b2)) + (-q - b2);
    const float lo = ((s1e + s2e) - qe) - kf * B2G_PIO256_3;
    const float rh = s2 + lo;
    const float rl = lo - (rh - s2);
    // sin r, cos r
    const float r2 = rh * rh;
    const float ts = (rh * r2) * (-0x1.555556p-3f + 0x1.111112p-7f * r2);
    const float sh = rh;
    const float sl = rl + ts;
    const float pl = fmaf(rh, rh, -r2);
    const float uh = 0.5f * r2;
    const float ul = 0.5f * pl + rh * rl;
    const float w = (r2 * r2) * 0x1.555556p-5f;
    const float ch = 1.0f - uh;
    const float b3 = ch - 1.0f;
    const float che = (1.0f - (ch - b3)) + (-uh - b3);
    const float cl = che + (w - ul);
    // table (one 16-byte row: S high, S low, C high, C low)
#ifdef __CUDA_ARCH__
    const float4 T = reinterpret_cast<const float4*>(kTrigTableDev)[idx];
    const float Sh = T.x, Sl = T.y, Ch = T.z, Cl = T.w;
#else
    const float* T = TrigTable() + 4 * idx;
    const float Sh = T[0], Sl = T[1], Ch = T[2], Cl = T[3];
#endif
    // sin x = S cos r + C sin r
    const float a1 = Sh * ch;
    const float a1l = fmaf(Sh, ch, -a1) + (Sh * cl + Sl * ch);
    const float a2 = Ch * sh;
    const float a2l = fmaf(Ch, sh, -a2) + (Ch * sl + Cl * sh);
    const float sa = a1 + a2;
    const float b4 = sa - a1;
    const float sae = (a1 - (sa - b4)) + (a2 - b4);
    // cos x = C cos r - S sin r
    const float c1 = Ch * ch;
    const float c1l = fmaf(Ch, ch, -c1) + (Ch * cl + Cl * ch);
    const float P = Sh * sh;
    const float c2 = -P;
    const float c2l = -fmaf(Sh, sh, -P) - (Sh * sl + Sl * sh);
    const float ca = c1 + c2;
    const float b5 = ca - c1;
    const float cae = (c1 - (ca - b5)) + (c2 - b5);
    *s_out = sa + ((sae + a1l) + a2l);
    *c_out = ca + ((cae + c1l) + c2l);
}

// ------------------------------------------------------------------ vectors (Common/b2Math.h)
struct Vec2 { float x, y; };
B2G_HD Vec2 V(float x, float y) { Vec2 r; r.x = x; r.y = y; return r; }
B2G_HD Vec2 operator+(Vec2 a, Vec2 b) { return V(a.x + b.x, a.y + b.y); }
B2G_HD Vec2 operator-(Vec2 a, Vec2 b) { return V(a.x - b.x, a.y - b.y); }
B2G_HD Vec2 operator-(Vec2 a) { return V(-a.x, -a.y); }
B2G_HD Vec2 operator*(float s, Vec2 a) { return V(s * a.x, s * a.y); }
B2G_HD float Dot(Vec2 a, Vec2 b) { return a.x * b.x + a.y * b.y; }
B2G_HD float Cross(Vec2 a, Vec2 b) { return a.x * b.y - a.y * b.x; }
B2G_HD Vec2 Cross(Vec2 a, float s) { return V(s * a.y, -s * a.x); }
B2G_HD Vec2 Cross(float s, Vec2 a) { return V(-s * a.y, s * a.x); }
B2G_HD float LengthSq(Vec2 a) { return a.x * a.x + a.y * a.y; }
B2G_HD float Length(Vec2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
B2G_HD float DistanceSq(Vec2 a, Vec2 b) { Vec2 c = a - b; return Dot(c, c); }
B2G_HD float Dist(Vec2 a, Vec2 b) { return Length(a - b); }
B2G_HD float Normalize(Vec2& v)
{
    float len = Length(v);
    if (len < kEpsilon) return 0.0f;
    float inv = 1.0f / len;
    v.x *= inv;
    v.y *= inv;
    return len;
}
// Ternary min/max with the reference's operand order (signed zeros and NaNs behave identically).
B2G_HD float Minf(float a, float b) { return a < b ? a : b; }
B2G_HD float Maxf(float a, float b) { return a > b ? a : b; }
B2G_HD int Mini(int a, int b) { return a < b ? a : b; }
B2G_HD int Maxi(int a, int b) { return a > b ? a : b; }
B2G_HD float Absf(float a) { return a > 0.0f ? a : -a; }
B2G_HD float Clampf(float a, float lo, float hi) { return Maxf(lo, Minf(a, hi)); }
B2G_HD Vec2 Min(Vec2 a, Vec2 b) { return V(Minf(a.x, b.x), Minf(a.y, b.y)); }
B2G_HD Vec2 Max(Vec2 a, Vec2 b) { return V(Maxf(a.x, b.x), Maxf(a.y, b.y)); }

struct Rot { float s, c; };
B2G_HD Rot RotOf(float angle) { Rot q; SinCos(angle, &q.s, &q.c); return q; }
B2G_HD Vec2 Mul(Rot q, Vec2 v) { return V(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
B2G_HD Vec2 MulT(Rot q, Vec2 v) { return V(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
B2G_HD Rot MulT(Rot q, Rot r)
{
    Rot o;
    o.s = q.c * r.s - q.s * r.c;
    o.c = q.c * r.c + q.s * r.s;
    return o;
}
struct Xf { Vec2 p; Rot q; };
B2G_HD Vec2 Mul(const Xf& T, Vec2 v)
{
    return V((T.q.c * v.x - T.q.s * v.y) + T.p.x, (T.q.s * v.x + T.q.c * v.y) + T.p.y);
}
B2G_HD Vec2 MulT(const Xf& T, Vec2 v)
{
    float px = v.x - T.p.x, py = v.y - T.p.y;
    return V(T.q.c * px + T.q.s * py, -T.q.s * px + T.q.c * py);
}
B2G_HD Xf MulT(const Xf& A, const Xf& B)
{
    Xf C;
    C.q = MulT(A.q, B.q);
    C.p = MulT(A.q, B.p - A.p);
    return C;
}

struct Sweep { Vec2 localCenter, c0, c; float a0, a, alpha0; };
// b2Sweep::GetTransform / Advance / Normalize (Common/b2Math.h:690-720)
B2G_HD void SweepXf(const Sweep& s, Xf* xf, float beta)
{
    xf->p = (1.0f - beta) * s.c0 + beta * s.c;
    float angle = (1.0f - beta) * s.a0 + beta * s.a;
    xf->q = RotOf(angle);
    xf->p = xf->p - Mul(xf->q, s.localCenter);
}
B2G_HD void SweepAdvance(Sweep& s, float alpha)
{
    float beta = (alpha - s.alpha0) / (1.0f - s.alpha0);
    s.c0 = s.c0 + beta * (s.c - s.c0);
    s.a0 += beta * (s.a - s.a0);
    s.alpha0 = alpha;
}
B2G_HD void SweepNormalize(Sweep& s)
{
    float twoPi = 2.0f * kPi;
    float d = twoPi * floorf(s.a0 / twoPi);
    s.a0 -= d;
    s.a -= d;
}

// Axis-aligned box as float4 {lower.x, lower.y, upper.x, upper.y}.
B2G_HD bool Overlap(float4 a, float4 b)
{
    // b2TestOverlap (Collision/b2Collision.h:246-259) computes b.lower - a.upper and a.lower - b.upper;
    // the sign of an IEEE difference equals the comparison, so this is the same predicate.
    if (b.x - a.z > 0.0f || b.y - a.w > 0.0f) return false;
    if (a.x - b.z > 0.0f || a.y - b.w > 0.0f) return false;
    return true;
}
B2G_HD bool Contains(float4 outer, float4 in)
{
    return outer.x <= in.x && outer.y <= in.y && in.z <= outer.z && in.w <= outer.w;
}
B2G_HD float4 Combine(float4 a, float4 b)
{
    float4 o;
    o.x = Minf(a.x, b.x); o.y = Minf(a.y, b.y);
    o.z = Maxf(a.z, b.z); o.w = Maxf(a.w, b.w);
    return o;
}

// ------------------------------------------------------------------ shapes
enum ShapeType { kCircle = 0, kEdge = 1, kPolygon = 2 };
// Shape geometry in one record. Circle: v[0] = center. Edge: v[0] = vertex1, v[1] = vertex2,
// v[2] = vertex0, v[3] = vertex3, hasV0/hasV3 flags. Polygon: count vertices and normals, centroid.
struct Shape {
    int type;
    int count;
    int hasV0, hasV3;
    float radius;
    int chain;     // an edge that is a chain's child (b2ChainShape::GetChildEdge): 1 the first, 2 a next one
    float pad[2];
    Vec2 centroid;
    Vec2 v[kMaxPolyVerts];
    Vec2 n[kMaxPolyVerts];
};

B2G_HD void PolygonSetAsBox(Shape& s, float hx, float hy)
{
    s.type = kPolygon; s.radius = kPolygonRadius; s.count = 4; s.hasV0 = 0; s.hasV3 = 0;
    s.v[0] = V(-hx, -hy); s.v[1] = V(hx, -hy); s.v[2] = V(hx, hy); s.v[3] = V(-hx, hy);
    s.n[0] = V(0.0f, -1.0f); s.n[1] = V(1.0f, 0.0f); s.n[2] = V(0.0f, 1.0f); s.n[3] = V(-1.0f, 0.0f);
    s.centroid = V(0.0f, 0.0f);
}

// b2PolygonShape::SetAsBox(hx, hy, center, angle) (Collision/Shapes/b2PolygonShape.cpp:47-70)
B2G_HD void PolygonSetAsBox(Shape& s, float hx, float hy, Vec2 center, float angle)
{
    PolygonSetAsBox(s, hx, hy);
    s.centroid = center;
    Xf xf;
    xf.p = center;
    xf.q = RotOf(angle);
    for (int i = 0; i < 4; ++i) {
        s.v[i] = Mul(xf, s.v[i]);
        s.n[i] = Mul(xf.q, s.n[i]);
    }
}

// b2PolygonShape::Set (Collision/Shapes/b2PolygonShape.cpp:119-252): weld points closer than
// sqrt(0.5*slop), gift-wrap the hull from the right-most (then lowest) point, edge normals, area
// centroid of the triangle fan from the origin (ComputeCentroid, :77-117).
B2G_HD void PolygonSet(Shape& s, const Vec2* points, int count)
{
    if (count < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    int n = Mini(count, kMaxPolyVerts);
    Vec2 ps[kMaxPolyVerts];
    int uniq = 0;
    for (int i = 0; i < n; ++i) {
        bool keep = true;
        for (int j = 0; j < uniq; ++j)
            if (DistanceSq(points[i], ps[j]) < 0.5f * kLinearSlop) { keep = false; break; }
        if (keep) ps[uniq++] = points[i];
    }
    n = uniq;
    if (n < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    int i0 = 0;
    float x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        float x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
    }
    int hull[kMaxPolyVerts];
    int m = 0, ih = i0;
    for (;;) {
        hull[m] = ih;
        int ie = 0;
        for (int j = 1; j < n; ++j) {
            if (ie == ih) { ie = j; continue; }
            Vec2 r = ps[ie] - ps[hull[m]];
            Vec2 v = ps[j] - ps[hull[m]];
            float c = Cross(r, v);
            if (c < 0.0f) ie = j;
            if (c == 0.0f && LengthSq(v) > LengthSq(r)) ie = j;
        }
        ++m;
        ih = ie;
        if (ie == i0 || m == kMaxPolyVerts) break;
    }
    if (m < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    s.type = kPolygon; s.radius = kPolygonRadius; s.count = m; s.hasV0 = 0; s.hasV3 = 0;
    for (int i = 0; i < m; ++i) s.v[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        int i2 = i + 1 < m ? i + 1 : 0;
        s.n[i] = Cross(s.v[i2] - s.v[i], 1.0f);
        Normalize(s.n[i]);
    }
    Vec2 c = V(0.0f, 0.0f);
    float area = 0.0f;
    const float inv3 = 1.0f / 3.0f;
    for (int i = 0; i < m; ++i) {
        Vec2 p2 = s.v[i], p3 = i + 1 < m ? s.v[i + 1] : s.v[0];
        Vec2 p1 = V(0.0f, 0.0f);
        float D = Cross(p2 - p1, p3 - p1);
        float tri = 0.5f * D;
        area += tri;
        c = c + (tri * inv3) * (p1 + p2 + p3);
    }
    float invArea = 1.0f / area;
    c.x *= invArea;
    c.y *= invArea;
    s.centroid = c;
}

struct MassData { float mass; Vec2 center; float I; };

// ComputeMass: polygon (b2PolygonShape.cpp:361-437), circle (b2CircleShape.cpp:95-101), edge (b2EdgeShape.cpp:132-138)
B2G_HD void ComputeMass(const Shape& s, float density, MassData* md)
{
    if (s.type == kCircle) {
        md->mass = density * kPi * s.radius * s.radius;
        md->center = s.v[0];
        md->I = md->mass * (0.5f * s.radius * s.radius + Dot(s.v[0], s.v[0]));
        return;
    }
    if (s.type == kEdge) {
        md->mass = 0.0f;
        md->center = 0.5f * (s.v[0] + s.v[1]);
        md->I = 0.0f;
        return;
    }
    Vec2 center = V(0.0f, 0.0f);
    float area = 0.0f, I = 0.0f;
    Vec2 ref = V(0.0f, 0.0f);
    for (int i = 0; i < s.count; ++i) ref = ref + s.v[i];
    float invCount = 1.0f / s.count;
    ref.x *= invCount;
    ref.y *= invCount;
    const float k_inv3 = 1.0f / 3.0f;
    for (int i = 0; i < s.count; ++i) {
        Vec2 e1 = s.v[i] - ref;
        Vec2 e2 = i + 1 < s.count ? s.v[i + 1] - ref : s.v[0] - ref;
        float D = Cross(e1, e2);
        float tri = 0.5f * D;
        area += tri;
        center = center + (tri * k_inv3) * (e1 + e2);
        float intx2 = e1.x * e1.x + e2.x * e1.x + e2.x * e2.x;
        float inty2 = e1.y * e1.y + e2.y * e1.y + e2.y * e2.y;
        I += (0.25f * k_inv3 * D) * (intx2 + inty2);
    }
    md->mass = density * area;
    float invArea = 1.0f / area;
    center.x *= invArea;
    center.y *= invArea;
    md->center = center + ref;
    md->I = density * I;
    md->I += md->mass * (Dot(md->center, md->center) - Dot(center, center));
}

// ComputeAABB: polygon (b2PolygonShape.cpp:342-359), circle (b2CircleShape.cpp:86-93), edge (b2EdgeShape.cpp:118-130);
// a chain's child edge has no radius in its box (b2ChainShape.cpp:171-187)
B2G_HD float4 ComputeAABB(const Shape& s, const Xf& xf)
{
    float4 o;
    if (s.type == kCircle) {
        Vec2 p = xf.p + Mul(xf.q, s.v[0]);
        o.x = p.x - s.radius; o.y = p.y - s.radius; o.z = p.x + s.radius; o.w = p.y + s.radius;
        return o;
    }
    Vec2 lower, upper;
    if (s.type == kEdge) {
        Vec2 a = Mul(xf, s.v[0]), b = Mul(xf, s.v[1]);
        lower = Min(a, b);
        upper = Max(a, b);
        if (s.chain) {
            o.x = lower.x; o.y = lower.y; o.z = upper.x; o.w = upper.y;
            return o;
        }
    } else {
        lower = Mul(xf, s.v[0]);
        upper = lower;
        for (int i = 1; i < s.count; ++i) {
            Vec2 v = Mul(xf, s.v[i]);
            lower = Min(lower, v);
            upper = Max(upper, v);
        }
    }
    o.x = lower.x - s.radius; o.y = lower.y - s.radius;
    o.z = upper.x + s.radius; o.w = upper.y + s.radius;
    return o;
}

// ------------------------------------------------------------------ manifolds (Collision/b2Collision.h)
// Contact feature ids packed as b2ContactID::key: indexA | indexB<<8 | typeA<<16 | typeB<<24.
enum { kFeatVertex = 0, kFeatFace = 1 };
B2G_HD uint32_t MakeId(int ia, int ib, int ta, int tb)
{
    return (uint32_t)(ia & 0xff) | ((uint32_t)(ib & 0xff) << 8) | ((uint32_t)(ta & 0xff) << 16) |
           ((uint32_t)(tb & 0xff) << 24);
}
B2G_HD uint32_t IdFlip(uint32_t id)
{
    return ((id >> 8) & 0xff) | ((id & 0xff) << 8) | (((id >> 24) & 0xff) << 16) | (((id >> 16) & 0xff) << 24);
}

enum ManifoldType { kCircles = 0, kFaceA = 1, kFaceB = 2 };
struct MPoint { Vec2 lp; float ni, ti; uint32_t id; };
struct Manifold {
    MPoint p[2];
    Vec2 localNormal, localPoint;
    int type, count;
};
struct WorldManifold { Vec2 normal; Vec2 pts[2]; float sep[2]; };

// b2WorldManifold::Initialize (Collision/b2Collision.cpp:22-87)
B2G_HD void WorldManifoldInit(WorldManifold* wm, const Manifold& m, const Xf& xfA, float rA, const Xf& xfB, float rB)
{
    if (m.count == 0) return;
    if (m.type == kCircles) {
        wm->normal = V(1.0f, 0.0f);
        Vec2 pA = Mul(xfA, m.localPoint), pB = Mul(xfB, m.p[0].lp);
        if (DistanceSq(pA, pB) > kEpsilon * kEpsilon) {
            wm->normal = pB - pA;
            Normalize(wm->normal);
        }
        Vec2 cA = pA + rA * wm->normal, cB = pB - rB * wm->normal;
        wm->pts[0] = 0.5f * (cA + cB);
        wm->sep[0] = Dot(cB - cA, wm->normal);
    } else if (m.type == kFaceA) {
        wm->normal = Mul(xfA.q, m.localNormal);
        Vec2 plane = Mul(xfA, m.localPoint);
        for (int i = 0; i < m.count; ++i) {
            Vec2 clip = Mul(xfB, m.p[i].lp);
            Vec2 cA = clip + (rA - Dot(clip - plane, wm->normal)) * wm->normal;
            Vec2 cB = clip - rB * wm->normal;
            wm->pts[i] = 0.5f * (cA + cB);
            wm->sep[i] = Dot(cB - cA, wm->normal);
        }
    } else {
        wm->normal = Mul(xfB.q, m.localNormal);
        Vec2 plane = Mul(xfB, m.localPoint);
        for (int i = 0; i < m.count; ++i) {
            Vec2 clip = Mul(xfA, m.p[i].lp);
            Vec2 cB = clip + (rB - Dot(clip - plane, wm->normal)) * wm->normal;
            Vec2 cA = clip - rA * wm->normal;
            wm->pts[i] = 0.5f * (cA + cB);
            wm->sep[i] = Dot(cA - cB, wm->normal);
        }
        wm->normal = -wm->normal;
    }
}

struct ClipV { Vec2 v; uint32_t id; };

// b2ClipSegmentToLine (Collision/b2Collision.cpp:204-235), Sutherland-Hodgman against one plane.
B2G_HD int ClipSegment(ClipV out[2], const ClipV in[2], Vec2 normal, float offset, int vertexIndexA)
{
    int n = 0;
    float d0 = Dot(normal, in[0].v) - offset;
    float d1 = Dot(normal, in[1].v) - offset;
    if (d0 <= 0.0f) out[n++] = in[0];
    if (d1 <= 0.0f) out[n++] = in[1];
    if (d0 * d1 < 0.0f) {
        float interp = d0 / (d0 - d1);
        out[n].v = in[0].v + interp * (in[1].v - in[0].v);
        out[n].id = MakeId(vertexIndexA, (in[0].id >> 8) & 0xff, kFeatVertex, kFeatFace);
        ++n;
    }
    return n;
}

// b2CollideCircles (Collision/b2CollideCircle.cpp:25-51)
B2G_HD void CollideCircles(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB)
{
    m->count = 0;
    Vec2 pA = Mul(xfA, a.v[0]), pB = Mul(xfB, b.v[0]);
    Vec2 d = pB - pA;
    float radius = a.radius + b.radius;
    if (Dot(d, d) > radius * radius) return;
    m->type = kCircles;
    m->localPoint = a.v[0];
    m->localNormal = V(0.0f, 0.0f);
    m->count = 1;
    m->p[0].lp = b.v[0];
    m->p[0].id = 0;
}

// b2CollidePolygonAndCircle (Collision/b2CollideCircle.cpp:53-154)
B2G_HD void CollidePolygonAndCircle(Manifold* m, const Shape& poly, const Xf& xfA, const Shape& circ, const Xf& xfB)
{
    m->count = 0;
    Vec2 cLocal = MulT(xfA, Mul(xfB, circ.v[0]));
    int normalIndex = 0;
    float separation = -kMaxFloat;
    float radius = poly.radius + circ.radius;
    for (int i = 0; i < poly.count; ++i) {
        float s = Dot(poly.n[i], cLocal - poly.v[i]);
        if (s > radius) return;
        if (s > separation) { separation = s; normalIndex = i; }
    }
    int i1 = normalIndex, i2 = i1 + 1 < poly.count ? i1 + 1 : 0;
    Vec2 v1 = poly.v[i1], v2 = poly.v[i2];
    m->p[0].lp = circ.v[0];
    m->p[0].id = 0;
    if (separation < kEpsilon) {
        m->count = 1; m->type = kFaceA;
        m->localNormal = poly.n[normalIndex];
        m->localPoint = 0.5f * (v1 + v2);
        return;
    }
    float u1 = Dot(cLocal - v1, v2 - v1);
    float u2 = Dot(cLocal - v2, v1 - v2);
    if (u1 <= 0.0f) {
        if (DistanceSq(cLocal, v1) > radius * radius) return;
        m->count = 1; m->type = kFaceA;
        m->localNormal = cLocal - v1;
        Normalize(m->localNormal);
        m->localPoint = v1;
    } else if (u2 <= 0.0f) {
        if (DistanceSq(cLocal, v2) > radius * radius) return;
        m->count = 1; m->type = kFaceA;
        m->localNormal = cLocal - v2;
        Normalize(m->localNormal);
        m->localPoint = v2;
    } else {
        Vec2 faceCenter = 0.5f * (v1 + v2);
        if (Dot(cLocal - faceCenter, poly.n[i1]) > radius) return;
        m->count = 1; m->type = kFaceA;
        m->localNormal = poly.n[i1];
        m->localPoint = faceCenter;
    }
}

// b2FindMaxSeparation (Collision/b2CollidePolygon.cpp:28-67)
B2G_HD float MaxSeparation(int* edge, const Shape& p1, const Xf& xf1, const Shape& p2, const Xf& xf2)
{
    Xf xf = MulT(xf2, xf1);
    int best = 0;
    float maxSep = -kMaxFloat;
    for (int i = 0; i < p1.count; ++i) {
        Vec2 n = Mul(xf.q, p1.n[i]);
        Vec2 v1 = Mul(xf, p1.v[i]);
        float si = kMaxFloat;
        for (int j = 0; j < p2.count; ++j) {
            float sij = Dot(n, p2.v[j] - v1);
            if (sij < si) si = sij;
        }
        if (si > maxSep) { maxSep = si; best = i; }
    }
    *edge = best;
    return maxSep;
}

// b2CollidePolygons (Collision/b2CollidePolygon.cpp:121-239) with b2FindIncidentEdge (:69-110)
B2G_HDNI void CollidePolygons(Manifold* m, const Shape& polyA, const Xf& xfA, const Shape& polyB, const Xf& xfB)
{
    m->count = 0;
    float totalRadius = polyA.radius + polyB.radius;
    int edgeA = 0;
    float sepA = MaxSeparation(&edgeA, polyA, xfA, polyB, xfB);
    if (sepA > totalRadius) return;
    int edgeB = 0;
    float sepB = MaxSeparation(&edgeB, polyB, xfB, polyA, xfA);
    if (sepB > totalRadius) return;
    const Shape* poly1;
    const Shape* poly2;
    Xf xf1, xf2;
    int edge1;
    bool flip;
    const float k_tol = 0.1f * kLinearSlop;
    if (sepB > sepA + k_tol) {
        poly1 = &polyB; poly2 = &polyA; xf1 = xfB; xf2 = xfA; edge1 = edgeB; m->type = kFaceB; flip = true;
    } else {
        poly1 = &polyA; poly2 = &polyB; xf1 = xfA; xf2 = xfB; edge1 = edgeA; m->type = kFaceA; flip = false;
    }
    ClipV inc[2];
    {
        Vec2 normal1 = MulT(xf2.q, Mul(xf1.q, poly1->n[edge1]));
        int index = 0;
        float minDot = kMaxFloat;
        for (int i = 0; i < poly2->count; ++i) {
            float dot = Dot(normal1, poly2->n[i]);
            if (dot < minDot) { minDot = dot; index = i; }
        }
        int i1 = index, i2 = i1 + 1 < poly2->count ? i1 + 1 : 0;
        inc[0].v = Mul(xf2, poly2->v[i1]);
        inc[0].id = MakeId(edge1, i1, kFeatFace, kFeatVertex);
        inc[1].v = Mul(xf2, poly2->v[i2]);
        inc[1].id = MakeId(edge1, i2, kFeatFace, kFeatVertex);
    }
    int count1 = poly1->count;
    int iv1 = edge1, iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
    Vec2 v11 = poly1->v[iv1], v12 = poly1->v[iv2];
    Vec2 localTangent = v12 - v11;
    Normalize(localTangent);
    Vec2 localNormal = Cross(localTangent, 1.0f);
    Vec2 planePoint = 0.5f * (v11 + v12);
    Vec2 tangent = Mul(xf1.q, localTangent);
    Vec2 normal = Cross(tangent, 1.0f);
    v11 = Mul(xf1, v11);
    v12 = Mul(xf1, v12);
    float frontOffset = Dot(normal, v11);
    float sideOffset1 = -Dot(tangent, v11) + totalRadius;
    float sideOffset2 = Dot(tangent, v12) + totalRadius;
    ClipV c1[2], c2[2];
    if (ClipSegment(c1, inc, -tangent, sideOffset1, iv1) < 2) return;
    if (ClipSegment(c2, c1, tangent, sideOffset2, iv2) < 2) return;
    m->localNormal = localNormal;
    m->localPoint = planePoint;
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = Dot(normal, c2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            m->p[pc].lp = MulT(xf2, c2[i].v);
            m->p[pc].id = flip ? IdFlip(c2[i].id) : c2[i].id;
            ++pc;
        }
    }
    m->count = pc;
}

// b2CollideEdgeAndCircle (Collision/b2CollideEdge.cpp:29-147)
B2G_HD void CollideEdgeAndCircle(Manifold* m, const Shape& edge, const Xf& xfA, const Shape& circ, const Xf& xfB)
{
    m->count = 0;
    Vec2 Q = MulT(xfA, Mul(xfB, circ.v[0]));
    Vec2 A = edge.v[0], B = edge.v[1];
    Vec2 e = B - A;
    float u = Dot(e, B - Q);
    float v = Dot(e, Q - A);
    float radius = edge.radius + circ.radius;
    m->p[0].lp = circ.v[0];
    if (v <= 0.0f) {
        Vec2 d = Q - A;
        if (Dot(d, d) > radius * radius) return;
        if (edge.hasV0) {
            Vec2 e1 = A - edge.v[2];
            if (Dot(e1, A - Q) > 0.0f) return;
        }
        m->count = 1; m->type = kCircles;
        m->localNormal = V(0.0f, 0.0f);
        m->localPoint = A;
        m->p[0].id = MakeId(0, 0, kFeatVertex, kFeatVertex);
        return;
    }
    if (u <= 0.0f) {
        Vec2 d = Q - B;
        if (Dot(d, d) > radius * radius) return;
        if (edge.hasV3) {
            Vec2 e2 = edge.v[3] - B;
            if (Dot(e2, Q - B) > 0.0f) return;
        }
        m->count = 1; m->type = kCircles;
        m->localNormal = V(0.0f, 0.0f);
        m->localPoint = B;
        m->p[0].id = MakeId(1, 0, kFeatVertex, kFeatVertex);
        return;
    }
    float den = Dot(e, e);
    Vec2 P = (1.0f / den) * (u * A + v * B);
    Vec2 d = Q - P;
    if (Dot(d, d) > radius * radius) return;
    Vec2 n = V(-e.y, e.x);
    if (Dot(n, Q - A) < 0.0f) n = V(-n.x, -n.y);
    Normalize(n);
    m->count = 1; m->type = kFaceA;
    m->localNormal = n;
    m->localPoint = A;
    m->p[0].id = MakeId(0, 0, kFeatFace, kFeatVertex);
}

// b2EPCollider::Collide (Collision/b2CollideEdge.cpp:230-620) with ComputeEdgeSeparation (:622-639)
// and ComputePolygonSeparation (:641-692): edge versus polygon honouring ghost vertices.
B2G_HDNI void CollideEdgeAndPolygon(Manifold* m, const Shape& edge, const Xf& xfA, const Shape& poly, const Xf& xfB)
{
    Xf xf = MulT(xfA, xfB);
    Vec2 centroidB = Mul(xf, poly.centroid);
    Vec2 v0 = edge.v[2], v1 = edge.v[0], v2 = edge.v[1], v3 = edge.v[3];
    bool hasV0 = edge.hasV0 != 0, hasV3 = edge.hasV3 != 0;
    Vec2 e1 = v2 - v1;
    Normalize(e1);
    Vec2 n0 = V(0.0f, 0.0f), n2 = V(0.0f, 0.0f);
    Vec2 n1 = V(e1.y, -e1.x);
    float off1 = Dot(n1, centroidB - v1), off0 = 0.0f, off2 = 0.0f;
    bool convex1 = false, convex2 = false;
    if (hasV0) {
        Vec2 e0 = v1 - v0;
        Normalize(e0);
        n0 = V(e0.y, -e0.x);
        convex1 = Cross(e0, e1) >= 0.0f;
        off0 = Dot(n0, centroidB - v0);
    }
    if (hasV3) {
        Vec2 e2 = v3 - v2;
        Normalize(e2);
        n2 = V(e2.y, -e2.x);
        convex2 = Cross(e1, e2) > 0.0f;
        off2 = Dot(n2, centroidB - v2);
    }
    bool front;
    Vec2 normal, lower, upper;
    if (hasV0 && hasV3) {
        if (convex1 && convex2) {
            front = off0 >= 0.0f || off1 >= 0.0f || off2 >= 0.0f;
            if (front) { normal = n1; lower = n0; upper = n2; } else { normal = -n1; lower = -n1; upper = -n1; }
        } else if (convex1) {
            front = off0 >= 0.0f || (off1 >= 0.0f && off2 >= 0.0f);
            if (front) { normal = n1; lower = n0; upper = n1; } else { normal = -n1; lower = -n2; upper = -n1; }
        } else if (convex2) {
            front = off2 >= 0.0f || (off0 >= 0.0f && off1 >= 0.0f);
            if (front) { normal = n1; lower = n1; upper = n2; } else { normal = -n1; lower = -n1; upper = -n0; }
        } else {
            front = off0 >= 0.0f && off1 >= 0.0f && off2 >= 0.0f;
            if (front) { normal = n1; lower = n1; upper = n1; } else { normal = -n1; lower = -n2; upper = -n0; }
        }
    } else if (hasV0) {
        if (convex1) {
            front = off0 >= 0.0f || off1 >= 0.0f;
            if (front) { normal = n1; lower = n0; upper = -n1; } else { normal = -n1; lower = n1; upper = -n1; }
        } else {
            front = off0 >= 0.0f && off1 >= 0.0f;
            if (front) { normal = n1; lower = n1; upper = -n1; } else { normal = -n1; lower = n1; upper = -n0; }
        }
    } else if (hasV3) {
        if (convex2) {
            front = off1 >= 0.0f || off2 >= 0.0f;
            if (front) { normal = n1; lower = -n1; upper = n2; } else { normal = -n1; lower = -n1; upper = n1; }
        } else {
            front = off1 >= 0.0f && off2 >= 0.0f;
            if (front) { normal = n1; lower = -n1; upper = n1; } else { normal = -n1; lower = -n2; upper = n1; }
        }
    } else {
        front = off1 >= 0.0f;
        if (front) { normal = n1; lower = -n1; upper = -n1; } else { normal = -n1; lower = n1; upper = n1; }
    }
    Vec2 pv[kMaxPolyVerts], pn[kMaxPolyVerts];
    int count = poly.count;
    for (int i = 0; i < count; ++i) {
        pv[i] = Mul(xf, poly.v[i]);
        pn[i] = Mul(xf.q, poly.n[i]);
    }
    float radius = 2.0f * kPolygonRadius;
    m->count = 0;
    // edge axis (type edgeA, always known)
    float edgeSep = FLT_MAX;
    for (int i = 0; i < count; ++i) {
        float s = Dot(normal, pv[i] - v1);
        if (s < edgeSep) edgeSep = s;
    }
    if (edgeSep > radius) return;
    // polygon axis: 0 unknown, 2 edgeB
    int polyType = 0, polyIndex = -1;
    float polySep = -FLT_MAX;
    {
        Vec2 perp = V(-normal.y, normal.x);
        for (int i = 0; i < count; ++i) {
            Vec2 n = -pn[i];
            float s1 = Dot(n, pv[i] - v1), s2 = Dot(n, pv[i] - v2);
            float s = Minf(s1, s2);
            if (s > radius) { polyType = 2; polyIndex = i; polySep = s; break; }
            if (Dot(n, perp) >= 0.0f) {
                if (Dot(n - upper, normal) < -kAngularSlop) continue;
            } else {
                if (Dot(n - lower, normal) < -kAngularSlop) continue;
            }
            if (s > polySep) { polyType = 2; polyIndex = i; polySep = s; }
        }
    }
    if (polyType != 0 && polySep > radius) return;
    const float k_relativeTol = 0.98f, k_absoluteTol = 0.001f;
    bool useEdge;
    if (polyType == 0) useEdge = true;
    else if (polySep > k_relativeTol * edgeSep + k_absoluteTol) useEdge = false;
    else useEdge = true;
    ClipV ie[2];
    int rfI1, rfI2;
    Vec2 rfV1, rfV2, rfN;
    if (useEdge) {
        m->type = kFaceA;
        int best = 0;
        float bestValue = Dot(normal, pn[0]);
        for (int i = 1; i < count; ++i) {
            float value = Dot(normal, pn[i]);
            if (value < bestValue) { bestValue = value; best = i; }
        }
        int i1 = best, i2 = i1 + 1 < count ? i1 + 1 : 0;
        ie[0].v = pv[i1]; ie[0].id = MakeId(0, i1, kFeatFace, kFeatVertex);
        ie[1].v = pv[i2]; ie[1].id = MakeId(0, i2, kFeatFace, kFeatVertex);
        if (front) { rfI1 = 0; rfI2 = 1; rfV1 = v1; rfV2 = v2; rfN = n1; }
        else { rfI1 = 1; rfI2 = 0; rfV1 = v2; rfV2 = v1; rfN = -n1; }
    } else {
        m->type = kFaceB;
        ie[0].v = v1; ie[0].id = MakeId(0, polyIndex, kFeatVertex, kFeatFace);
        ie[1].v = v2; ie[1].id = MakeId(0, polyIndex, kFeatVertex, kFeatFace);
        rfI1 = polyIndex;
        rfI2 = rfI1 + 1 < count ? rfI1 + 1 : 0;
        rfV1 = pv[rfI1]; rfV2 = pv[rfI2]; rfN = pn[rfI1];
    }
    Vec2 side1 = V(rfN.y, -rfN.x);
    Vec2 side2 = -side1;
    float sideOff1 = Dot(side1, rfV1), sideOff2 = Dot(side2, rfV2);
    ClipV c1[2], c2[2];
    if (ClipSegment(c1, ie, side1, sideOff1, rfI1) < 2) return;
    if (ClipSegment(c2, c1, side2, sideOff2, rfI2) < 2) return;
    if (useEdge) { m->localNormal = rfN; m->localPoint = rfV1; }
    else { m->localNormal = poly.n[rfI1]; m->localPoint = poly.v[rfI1]; }
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = Dot(rfN, c2[i].v - rfV1);
        if (separation <= radius) {
            if (useEdge) { m->p[pc].lp = MulT(xf, c2[i].v); m->p[pc].id = c2[i].id; }
            else { m->p[pc].lp = c2[i].v; m->p[pc].id = IdFlip(c2[i].id); }
            ++pc;
        }
    }
    m->count = pc;
}

// Dispatch on the contact's (A, B) shape types; the contact factory has already put the primary type
// in A (Dynamics/Contacts/b2Contact.cpp:40-100).
B2G_HD void Evaluate(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB)
{
    if (a.type == kCircle) CollideCircles(m, a, xfA, b, xfB);
    else if (a.type == kPolygon && b.type == kCircle) CollidePolygonAndCircle(m, a, xfA, b, xfB);
    else if (a.type == kPolygon) CollidePolygons(m, a, xfA, b, xfB);
    else if (b.type == kCircle) CollideEdgeAndCircle(m, a, xfA, b, xfB);
    else CollideEdgeAndPolygon(m, a, xfA, b, xfB);
}

// ------------------------------------------------------------------ GJK distance (Collision/b2Distance.cpp)
// ------------------------------------------------------------------ shape ray casts
// b2Shape::RayCast for one fixture (Collision/Shapes/b2CircleShape.cpp:49-84, b2EdgeShape.cpp:56-116,
// b2PolygonShape.cpp:270-340), segment p1 -> p2 with maxFraction, shape at transform xf. Returns
// whether the segment hits the shape, the fraction along it and the world normal.
B2G_HD bool RayCastShape(const Shape& sh, const Xf& xf, Vec2 p1, Vec2 p2, float maxFraction, float* fraction,
                         Vec2* normal)
{
    if (sh.type == kCircle) {
        const Vec2 position = xf.p + Mul(xf.q, sh.v[0]);
        const Vec2 s = p1 - position;
        const float b = Dot(s, s) - sh.radius * sh.radius;
        const Vec2 r = p2 - p1;
        const float c = Dot(s, r);
        const float rr = Dot(r, r);
        const float sigma = c * c - rr * b;
        if (sigma < 0.0f || rr < kEpsilon) return false;
        float a = -(c + sqrtf(sigma));
        if (0.0f <= a && a <= maxFraction * rr) {
            a /= rr;
            *fraction = a;
            Vec2 n = s + a * r;
            Normalize(n);
            *normal = n;
            return true;
        }
        return false;
    }
    const Vec2 q1 = MulT(xf.q, p1 - xf.p);
    const Vec2 q2 = MulT(xf.q, p2 - xf.p);
    const Vec2 d = q2 - q1;
    if (sh.type == kEdge) {
        const Vec2 v1 = sh.v[0], v2 = sh.v[1];
        const Vec2 e = v2 - v1;
        Vec2 n = V(e.y, -e.x);
        Normalize(n);
        const float numerator = Dot(n, v1 - q1);
        const float denominator = Dot(n, d);
        if (denominator == 0.0f) return false;
        const float t = numerator / denominator;
        if (t < 0.0f || maxFraction < t) return false;
        const Vec2 q = q1 + t * d;
        const Vec2 r = v2 - v1;
        const float rr = Dot(r, r);
        if (rr == 0.0f) return false;
        const float sEdge = Dot(q - v1, r) / rr;
        if (sEdge < 0.0f || 1.0f < sEdge) return false;
        *fraction = t;
        *normal = numerator > 0.0f ? -Mul(xf.q, n) : Mul(xf.q, n);
        return true;
    }
    float lower = 0.0f, upper = maxFraction;
    int index = -1;
    for (int i = 0; i < sh.count; ++i) {
        const float numerator = Dot(sh.n[i], sh.v[i] - q1);
        const float denominator = Dot(sh.n[i], d);
        if (denominator == 0.0f) {
            if (numerator < 0.0f) return false;
        } else if (denominator < 0.0f && numerator < lower * denominator) {
            lower = numerator / denominator;
            index = i;
        } else if (denominator > 0.0f && numerator < upper * denominator) {
            upper = numerator / denominator;
        }
        if (upper < lower) return false;
    }
    if (index >= 0) {
        *fraction = lower;
        *normal = Mul(xf.q, sh.n[index]);
        return true;
    }
    return false;
}

struct Proxy { const Vec2* v; int count; float radius; };
B2G_HD Proxy ProxyOf(const Shape& s)
{
    Proxy p;
    p.v = s.v;
    p.count = s.type == kCircle ? 1 : (s.type == kEdge ? 2 : s.count);
    p.radius = s.radius;
    return p;
}
B2G_HD int Support(const Proxy& p, Vec2 d)
{
    int best = 0;
    float bestValue = Dot(p.v[0], d);
    for (int i = 1; i < p.count; ++i) {
        float value = Dot(p.v[i], d);
        if (value > bestValue) { best = i; bestValue = value; }
    }
    return best;
}
struct SimplexCache { float metric; int count; int ia[3], ib[3]; };
struct SVert { Vec2 wA, wB, w; float a; int ia, ib; };

B2G_HD float SimplexMetric(const SVert* v, int count)
{
    if (count == 2) return Dist(v[0].w, v[1].w);
    if (count == 3) return Cross(v[1].w - v[0].w, v[2].w - v[0].w);
    return 0.0f;
}

// b2Distance (Collision/b2Distance.cpp:402-535) with b2Simplex ReadCache/Solve2/Solve3 (:94-400)
B2G_HDNI float Distance(Vec2* pA, Vec2* pB, SimplexCache* cache, const Proxy& A, const Xf& xfA, const Proxy& B,
                        const Xf& xfB, bool useRadii)
{
    SVert v[3];
    int count = cache->count;
    for (int i = 0; i < count; ++i) {
        v[i].ia = cache->ia[i]; v[i].ib = cache->ib[i];
        v[i].wA = Mul(xfA, A.v[v[i].ia]);
        v[i].wB = Mul(xfB, B.v[v[i].ib]);
        v[i].w = v[i].wB - v[i].wA;
        v[i].a = 0.0f;
    }
    if (count > 1) {
        float m1 = cache->metric, m2 = SimplexMetric(v, count);
        if (m2 < 0.5f * m1 || 2.0f * m1 < m2 || m2 < kEpsilon) count = 0;
    }
    if (count == 0) {
        v[0].ia = 0; v[0].ib = 0;
        v[0].wA = Mul(xfA, A.v[0]);
        v[0].wB = Mul(xfB, B.v[0]);
        v[0].w = v[0].wB - v[0].wA;
        v[0].a = 1.0f;
        count = 1;
    }
    int saveA[3], saveB[3];
    int iter = 0;
    while (iter < 20) {
        int saveCount = count;
        for (int i = 0; i < saveCount; ++i) { saveA[i] = v[i].ia; saveB[i] = v[i].ib; }
        if (count == 2) {
            Vec2 w1 = v[0].w, w2 = v[1].w;
            Vec2 e12 = w2 - w1;
            float d12_2 = -Dot(w1, e12);
            if (d12_2 <= 0.0f) { v[0].a = 1.0f; count = 1; }
            else {
                float d12_1 = Dot(w2, e12);
                if (d12_1 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; }
                else {
                    float inv = 1.0f / (d12_1 + d12_2);
                    v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; count = 2;
                }
            }
        } else if (count == 3) {
            Vec2 w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
            Vec2 e12 = w2 - w1;
            float d12_1 = Dot(w2, e12), d12_2 = -Dot(w1, e12);
            Vec2 e13 = w3 - w1;
            float d13_1 = Dot(w3, e13), d13_2 = -Dot(w1, e13);
            Vec2 e23 = w3 - w2;
            float d23_1 = Dot(w3, e23), d23_2 = -Dot(w2, e23);
            float n123 = Cross(e12, e13);
            float d123_1 = n123 * Cross(w2, w3);
            float d123_2 = n123 * Cross(w3, w1);
            float d123_3 = n123 * Cross(w1, w2);
            if (d12_2 <= 0.0f && d13_2 <= 0.0f) { v[0].a = 1.0f; count = 1; }
            else if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
                float inv = 1.0f / (d12_1 + d12_2);
                v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; count = 2;
            } else if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
                float inv = 1.0f / (d13_1 + d13_2);
                v[0].a = d13_1 * inv; v[2].a = d13_2 * inv; count = 2; v[1] = v[2];
            } else if (d12_1 <= 0.0f && d23_2 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; }
            else if (d13_1 <= 0.0f && d23_1 <= 0.0f) { v[2].a = 1.0f; count = 1; v[0] = v[2]; }
            else if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
                float inv = 1.0f / (d23_1 + d23_2);
                v[1].a = d23_1 * inv; v[2].a = d23_2 * inv; count = 2; v[0] = v[2];
            } else {
                float inv = 1.0f / (d123_1 + d123_2 + d123_3);
                v[0].a = d123_1 * inv; v[1].a = d123_2 * inv; v[2].a = d123_3 * inv; count = 3;
            }
        }
        if (count == 3) break;
        Vec2 d;
        if (count == 1) d = -v[0].w;
        else {
            Vec2 e12 = v[1].w - v[0].w;
            float sgn = Cross(e12, -v[0].w);
            d = sgn > 0.0f ? Cross(1.0f, e12) : Cross(e12, 1.0f);
        }
        if (LengthSq(d) < kEpsilon * kEpsilon) break;
        SVert& nv = v[count];
        nv.ia = Support(A, MulT(xfA.q, -d));
        nv.wA = Mul(xfA, A.v[nv.ia]);
        nv.ib = Support(B, MulT(xfB.q, d));
        nv.wB = Mul(xfB, B.v[nv.ib]);
        nv.w = nv.wB - nv.wA;
        ++iter;
        bool dup = false;
        for (int i = 0; i < saveCount; ++i)
            if (nv.ia == saveA[i] && nv.ib == saveB[i]) { dup = true; break; }
        if (dup) break;
        ++count;
    }
    Vec2 a, b;
    if (count == 1) { a = v[0].wA; b = v[0].wB; }
    else if (count == 2) {
        a = v[0].a * v[0].wA + v[1].a * v[1].wA;
        b = v[0].a * v[0].wB + v[1].a * v[1].wB;
    } else {
        a = v[0].a * v[0].wA + v[1].a * v[1].wA + v[2].a * v[2].wA;
        b = a;
    }
    float distance = Dist(a, b);
    cache->metric = SimplexMetric(v, count);
    cache->count = count;
    for (int i = 0; i < count; ++i) { cache->ia[i] = v[i].ia & 0xff; cache->ib[i] = v[i].ib & 0xff; }
    if (useRadii) {
        float rA = A.radius, rB = B.radius;
        if (distance > rA + rB && distance > kEpsilon) {
            distance -= rA + rB;
            Vec2 normal = b - a;
            Normalize(normal);
            a = a + rA * normal;
            b = b - rB * normal;
        } else {
            Vec2 p = 0.5f * (a + b);
            a = p;
            b = p;
            distance = 0.0f;
        }
    }
    *pA = a;
    *pB = b;
    return distance;
}

// ------------------------------------------------------------------ time of impact (Collision/b2TimeOfImpact.cpp)
enum { kToiUnknown = 0, kToiFailed = 1, kToiOverlapped = 2, kToiTouching = 3, kToiSeparated = 4 };
enum { kSepPoints = 0, kSepFaceA = 1, kSepFaceB = 2 };
struct SepFn {
    Proxy A, B;
    Sweep sa, sb;
    int type;
    Vec2 localPoint, axis;
};

// b2SeparationFunction::Initialize (b2TimeOfImpact.cpp:43-119)
B2G_HD float SepInit(SepFn& f, const SimplexCache& cache, float t1)
{
    Xf xfA, xfB;
    SweepXf(f.sa, &xfA, t1);
    SweepXf(f.sb, &xfB, t1);
    if (cache.count == 1) {
        f.type = kSepPoints;
        Vec2 pA = Mul(xfA, f.A.v[cache.ia[0]]), pB = Mul(xfB, f.B.v[cache.ib[0]]);
        f.axis = pB - pA;
        return Normalize(f.axis);
    }
    if (cache.ia[0] == cache.ia[1]) {
        f.type = kSepFaceB;
        Vec2 b1 = f.B.v[cache.ib[0]], b2 = f.B.v[cache.ib[1]];
        f.axis = Cross(b2 - b1, 1.0f);
        Normalize(f.axis);
        Vec2 normal = Mul(xfB.q, f.axis);
        f.localPoint = 0.5f * (b1 + b2);
        Vec2 pB = Mul(xfB, f.localPoint), pA = Mul(xfA, f.A.v[cache.ia[0]]);
        float s = Dot(pA - pB, normal);
        if (s < 0.0f) { f.axis = -f.axis; s = -s; }
        return s;
    }
    f.type = kSepFaceA;
    Vec2 a1 = f.A.v[cache.ia[0]], a2 = f.A.v[cache.ia[1]];
    f.axis = Cross(a2 - a1, 1.0f);
    Normalize(f.axis);
    Vec2 normal = Mul(xfA.q, f.axis);
    f.localPoint = 0.5f * (a1 + a2);
    Vec2 pA = Mul(xfA, f.localPoint), pB = Mul(xfB, f.B.v[cache.ib[0]]);
    float s = Dot(pB - pA, normal);
    if (s < 0.0f) { f.axis = -f.axis; s = -s; }
    return s;
}

// b2SeparationFunction::FindMinSeparation (b2TimeOfImpact.cpp:121-182)
B2G_HD float SepFindMin(const SepFn& f, int* iA, int* iB, float t)
{
    Xf xfA, xfB;
    SweepXf(f.sa, &xfA, t);
    SweepXf(f.sb, &xfB, t);
    if (f.type == kSepPoints) {
        *iA = Support(f.A, MulT(xfA.q, f.axis));
        *iB = Support(f.B, MulT(xfB.q, -f.axis));
        Vec2 pA = Mul(xfA, f.A.v[*iA]), pB = Mul(xfB, f.B.v[*iB]);
        return Dot(pB - pA, f.axis);
    }
    if (f.type == kSepFaceA) {
        Vec2 normal = Mul(xfA.q, f.axis);
        Vec2 pA = Mul(xfA, f.localPoint);
        *iA = -1;
        *iB = Support(f.B, MulT(xfB.q, -normal));
        Vec2 pB = Mul(xfB, f.B.v[*iB]);
        return Dot(pB - pA, normal);
    }
    Vec2 normal = Mul(xfB.q, f.axis);
    Vec2 pB = Mul(xfB, f.localPoint);
    *iB = -1;
    *iA = Support(f.A, MulT(xfA.q, -normal));
    Vec2 pA = Mul(xfA, f.A.v[*iA]);
    return Dot(pA - pB, normal);
}

// b2SeparationFunction::Evaluate (b2TimeOfImpact.cpp:184-232)
B2G_HD float SepEval(const SepFn& f, int iA, int iB, float t)
{
    Xf xfA, xfB;
    SweepXf(f.sa, &xfA, t);
    SweepXf(f.sb, &xfB, t);
    if (f.type == kSepPoints) {
        Vec2 pA = Mul(xfA, f.A.v[iA]), pB = Mul(xfB, f.B.v[iB]);
        return Dot(pB - pA, f.axis);
    }
    if (f.type == kSepFaceA) {
        Vec2 normal = Mul(xfA.q, f.axis);
        Vec2 pA = Mul(xfA, f.localPoint), pB = Mul(xfB, f.B.v[iB]);
        return Dot(pB - pA, normal);
    }
    Vec2 normal = Mul(xfB.q, f.axis);
    Vec2 pB = Mul(xfB, f.localPoint), pA = Mul(xfA, f.A.v[iA]);
    return Dot(pA - pB, normal);
}

// b2TimeOfImpact (b2TimeOfImpact.cpp:257-481): conservative advancement with a root finder that
// alternates bisection and secant steps; target separation max(slop, R - 3*slop) +- slop/4.
B2G_HDNI void TimeOfImpact(int* state, float* tOut, const Proxy& A, const Proxy& B, const Sweep& swA, const Sweep& swB,
                           float tMax)
{
    *state = kToiUnknown;
    *tOut = tMax;
    SepFn f;
    f.A = A; f.B = B;
    f.sa = swA; f.sb = swB;
    SweepNormalize(f.sa);
    SweepNormalize(f.sb);
    float totalRadius = A.radius + B.radius;
    float target = Maxf(kLinearSlop, totalRadius - 3.0f * kLinearSlop);
    float tolerance = 0.25f * kLinearSlop;
    float t1 = 0.0f;
    int iter = 0;
    SimplexCache cache;
    cache.count = 0;
    cache.metric = 0.0f;
    for (;;) {
        Xf xfA, xfB;
        SweepXf(f.sa, &xfA, t1);
        SweepXf(f.sb, &xfB, t1);
        Vec2 pa, pb;
        float distance = Distance(&pa, &pb, &cache, A, xfA, B, xfB, false);
        if (distance <= 0.0f) { *state = kToiOverlapped; *tOut = 0.0f; break; }
        if (distance < target + tolerance) { *state = kToiTouching; *tOut = t1; break; }
        SepInit(f, cache, t1);
        bool done = false;
        float t2 = tMax;
        int pushBackIter = 0;
        for (;;) {
            int iA, iB;
            float s2 = SepFindMin(f, &iA, &iB, t2);
            if (s2 > target + tolerance) { *state = kToiSeparated; *tOut = tMax; done = true; break; }
            if (s2 > target - tolerance) { t1 = t2; break; }
            float s1 = SepEval(f, iA, iB, t1);
            if (s1 < target - tolerance) { *state = kToiFailed; *tOut = t1; done = true; break; }
            if (s1 <= target + tolerance) { *state = kToiTouching; *tOut = t1; done = true; break; }
            int rootIter = 0;
            float a1 = t1, a2 = t2;
            for (;;) {
                float t;
                if (rootIter & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5f * (a1 + a2);
                ++rootIter;
                float s = SepEval(f, iA, iB, t);
                if (Absf(s - target) < tolerance) { t2 = t; break; }
                if (s > target) { a1 = t; s1 = s; } else { a2 = t; s2 = s; }
                if (rootIter == 50) break;
            }
            ++pushBackIter;
            if (pushBackIter == kMaxPolyVerts) break;
        }
        ++iter;
        if (done) break;
        if (iter == 20) { *state = kToiFailed; *tOut = t1; break; }
    }
}

} // namespace b2g
