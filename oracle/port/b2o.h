// Oracle (test infrastructure only): the project's CPU restatement of the Box2D 2.3.2 step
// (b2World::Step and everything below it) that the GPU path is checked against where the reference
// tree is not available. It is written index-based (no pointers, no allocators) but evaluates every
// floating-point expression in the same order as the reference, so that compiled with
// -ffp-contract=off it reproduces the reference bit for bit when it uses the same sin/cos.
//
// Citations are to the reference tree Regression/box2d-ref/Box2DRef/ (vendored Box2D 2.3.2).
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

extern "C" void b2o_sincosf(float x, float* s, float* c);

namespace b2o {

// Common/b2Settings.h:44-160
constexpr float kEpsilon = FLT_EPSILON;
constexpr float kMaxFloat = FLT_MAX;
constexpr float kPi = 3.14159265359f;
constexpr int kMaxManifoldPoints = 2;
constexpr int kMaxPolygonVertices = 8;
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

// Which sin/cos b2Rot::Set uses: libm (matches the reference on the same libc) or the project trig.
extern int g_trig_mode; // 0 = libm sinf/cosf, 1 = project b2o_sincosf

struct Vec2 { float x, y; };
inline Vec2 V(float x, float y) { Vec2 r; r.x = x; r.y = y; return r; }
inline Vec2 operator+(Vec2 a, Vec2 b) { return V(a.x + b.x, a.y + b.y); }
inline Vec2 operator-(Vec2 a, Vec2 b) { return V(a.x - b.x, a.y - b.y); }
inline Vec2 operator-(Vec2 a) { return V(-a.x, -a.y); }
inline Vec2 operator*(float s, Vec2 a) { return V(s * a.x, s * a.y); }
inline float Dot(Vec2 a, Vec2 b) { return a.x * b.x + a.y * b.y; }
inline float Cross(Vec2 a, Vec2 b) { return a.x * b.y - a.y * b.x; }
inline Vec2 Cross(Vec2 a, float s) { return V(s * a.y, -s * a.x); }
inline Vec2 Cross(float s, Vec2 a) { return V(-s * a.y, s * a.x); }
inline float LengthSq(Vec2 a) { return a.x * a.x + a.y * a.y; }
inline float Length(Vec2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
inline float DistanceSq(Vec2 a, Vec2 b) { Vec2 c = a - b; return Dot(c, c); }
inline float Distance(Vec2 a, Vec2 b) { return Length(a - b); }
// b2Vec2::Normalize (Common/b2Math.h:94-106)
inline float Normalize(Vec2& v)
{
    float len = Length(v);
    if (len < kEpsilon) return 0.0f;
    float inv = 1.0f / len;
    v.x *= inv;
    v.y *= inv;
    return len;
}
template <typename T> inline T Min(T a, T b) { return a < b ? a : b; }
template <typename T> inline T Max(T a, T b) { return a > b ? a : b; }
template <typename T> inline T Abs(T a) { return a > T(0) ? a : -a; }
template <typename T> inline T Clamp(T a, T lo, T hi) { return Max(lo, Min(a, hi)); }
inline Vec2 Min(Vec2 a, Vec2 b) { return V(Min(a.x, b.x), Min(a.y, b.y)); }
inline Vec2 Max(Vec2 a, Vec2 b) { return V(Max(a.x, b.x), Max(a.y, b.y)); }

struct Rot { float s, c; };
inline Rot RotOf(float angle)
{
    Rot q;
    if (g_trig_mode == 0) { q.s = sinf(angle); q.c = cosf(angle); }
    else b2o_sincosf(angle, &q.s, &q.c);
    return q;
}
inline Vec2 Mul(Rot q, Vec2 v) { return V(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
inline Vec2 MulT(Rot q, Vec2 v) { return V(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
inline Rot MulT(Rot q, Rot r)
{
    Rot o;
    o.s = q.c * r.s - q.s * r.c;
    o.c = q.c * r.c + q.s * r.s;
    return o;
}

struct Xf { Vec2 p; Rot q; };
inline Vec2 Mul(const Xf& T, Vec2 v)
{
    float x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
    float y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
    return V(x, y);
}
inline Vec2 MulT(const Xf& T, Vec2 v)
{
    float px = v.x - T.p.x;
    float py = v.y - T.p.y;
    return V(T.q.c * px + T.q.s * py, -T.q.s * px + T.q.c * py);
}
inline Xf MulT(const Xf& A, const Xf& B)
{
    Xf C;
    C.q = MulT(A.q, B.q);
    C.p = MulT(A.q, B.p - A.p);
    return C;
}

struct Sweep {
    Vec2 localCenter, c0, c;
    float a0, a, alpha0;
};
// b2Sweep::GetTransform / Advance / Normalize (Common/b2Math.h:690-720)
inline void SweepXf(const Sweep& s, Xf* xf, float beta)
{
    xf->p = (1.0f - beta) * s.c0 + beta * s.c;
    float angle = (1.0f - beta) * s.a0 + beta * s.a;
    xf->q = RotOf(angle);
    xf->p = xf->p - Mul(xf->q, s.localCenter);
}
inline void SweepAdvance(Sweep& s, float alpha)
{
    float beta = (alpha - s.alpha0) / (1.0f - s.alpha0);
    s.c0 = s.c0 + beta * (s.c - s.c0);
    s.a0 += beta * (s.a - s.a0);
    s.alpha0 = alpha;
}
inline void SweepNormalize(Sweep& s)
{
    float twoPi = 2.0f * kPi;
    float d = twoPi * floorf(s.a0 / twoPi);
    s.a0 -= d;
    s.a -= d;
}

struct AABB { Vec2 lo, hi; };
inline bool Overlap(const AABB& a, const AABB& b)
{
    Vec2 d1 = b.lo - a.hi, d2 = a.lo - b.hi;
    if (d1.x > 0.0f || d1.y > 0.0f) return false;
    if (d2.x > 0.0f || d2.y > 0.0f) return false;
    return true;
}
inline bool Contains(const AABB& outer, const AABB& in)
{
    return outer.lo.x <= in.lo.x && outer.lo.y <= in.lo.y && in.hi.x <= outer.hi.x && in.hi.y <= outer.hi.y;
}
inline AABB Combine(const AABB& a, const AABB& b)
{
    AABB o;
    o.lo = Min(a.lo, b.lo);
    o.hi = Max(a.hi, b.hi);
    return o;
}
inline float Perimeter(const AABB& a)
{
    float wx = a.hi.x - a.lo.x, wy = a.hi.y - a.lo.y;
    return 2.0f * (wx + wy);
}

// Shapes: Collision/Shapes/b2Shape.h (e_circle 0, e_edge 1, e_polygon 2)
enum ShapeType { kCircle = 0, kEdge = 1, kPolygon = 2 };
struct Shape {
    int type = kCircle;
    float radius = 0.0f;
    Vec2 p{0, 0};                    // circle center
    Vec2 v0{0, 0}, v1{0, 0}, v2{0, 0}, v3{0, 0};
    bool hasV0 = false, hasV3 = false; // edge
    int chain = 0;                     // edge that is a chain's child: 1 the first, 2 a next one
    int count = 0;
    Vec2 verts[kMaxPolygonVertices], normals[kMaxPolygonVertices];
    Vec2 centroid{0, 0};             // polygon
};
struct MassData { float mass; Vec2 center; float I; };

void PolygonSetAsBox(Shape& s, float hx, float hy);
void PolygonSetAsBox(Shape& s, float hx, float hy, Vec2 center, float angle);
void PolygonSet(Shape& s, const Vec2* pts, int count);
void ComputeMass(const Shape& s, float density, MassData* md);
void ComputeAABB(const Shape& s, const Xf& xf, AABB* out);

// Manifold: Collision/b2Collision.h:55-110. ids are the 4-byte b2ContactID packed little-endian
// (indexA | indexB<<8 | typeA<<16 | typeB<<24), the value b2ContactID::key holds.
enum { kFeatureVertex = 0, kFeatureFace = 1 };
inline uint32_t MakeId(int indexA, int indexB, int typeA, int typeB)
{
    return (uint32_t)(uint8_t)indexA | ((uint32_t)(uint8_t)indexB << 8) | ((uint32_t)(uint8_t)typeA << 16) |
           ((uint32_t)(uint8_t)typeB << 24);
}
inline int IdIndexA(uint32_t id) { return (int)(id & 0xff); }
inline int IdIndexB(uint32_t id) { return (int)((id >> 8) & 0xff); }
inline int IdTypeA(uint32_t id) { return (int)((id >> 16) & 0xff); }
inline int IdTypeB(uint32_t id) { return (int)((id >> 24) & 0xff); }
inline uint32_t IdFlip(uint32_t id) { return MakeId(IdIndexB(id), IdIndexA(id), IdTypeB(id), IdTypeA(id)); }

enum ManifoldType { kCircles = 0, kFaceA = 1, kFaceB = 2 };
struct ManifoldPoint { Vec2 localPoint; float normalImpulse, tangentImpulse; uint32_t id; };
struct Manifold {
    ManifoldPoint points[kMaxManifoldPoints];
    Vec2 localNormal, localPoint;
    int type;
    int pointCount;
};
struct WorldManifold { Vec2 normal; Vec2 points[2]; float separations[2]; };

void WorldManifoldInit(WorldManifold* wm, const Manifold* m, const Xf& xfA, float radiusA, const Xf& xfB, float radiusB);
void CollideCircles(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void CollidePolygonAndCircle(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void CollidePolygons(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void CollideEdgeAndCircle(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void CollideEdgeAndPolygon(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);

// Distance and time of impact: Collision/b2Distance.h, b2TimeOfImpact.h
struct DistanceProxy { const Vec2* verts; int count; float radius; };
void ProxyOf(DistanceProxy* p, const Shape& s);
struct SimplexCache { float metric; int count; uint8_t indexA[3], indexB[3]; };
struct DistanceOutput { Vec2 pointA, pointB; float distance; int iterations; };
void Distance(DistanceOutput* out, SimplexCache* cache, const DistanceProxy& pa, const Xf& xfA,
              const DistanceProxy& pb, const Xf& xfB, bool useRadii);
enum TOIState { kToiUnknown = 0, kToiFailed, kToiOverlapped, kToiTouching, kToiSeparated };
void TimeOfImpact(int* state, float* t, const DistanceProxy& pa, const DistanceProxy& pb, const Sweep& swA,
                  const Sweep& swB, float tMax);

} // namespace b2o
