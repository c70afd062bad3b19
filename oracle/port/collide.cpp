// Oracle (test infrastructure only): shapes, narrowphase, GJK distance and time of impact,
// restated from the reference Box2D 2.3.2 (paths relative to Regression/box2d-ref/Box2DRef/).
#include "b2o.h"

namespace b2o {

int g_trig_mode = 0;

// ---------------------------------------------------------------- shapes
// b2PolygonShape::SetAsBox (Collision/Shapes/b2PolygonShape.cpp:33-45)
void PolygonSetAsBox(Shape& s, float hx, float hy)
{
    s.type = kPolygon;
    s.radius = kPolygonRadius;
    s.count = 4;
    s.verts[0] = V(-hx, -hy); s.verts[1] = V(hx, -hy); s.verts[2] = V(hx, hy); s.verts[3] = V(-hx, hy);
    s.normals[0] = V(0.0f, -1.0f); s.normals[1] = V(1.0f, 0.0f); s.normals[2] = V(0.0f, 1.0f); s.normals[3] = V(-1.0f, 0.0f);
    s.centroid = V(0.0f, 0.0f);
}

// b2PolygonShape::SetAsBox with center and angle (Collision/Shapes/b2PolygonShape.cpp:47-70)
void PolygonSetAsBox(Shape& s, float hx, float hy, Vec2 center, float angle)
{
    PolygonSetAsBox(s, hx, hy);
    s.centroid = center;
    Xf xf;
    xf.p = center;
    xf.q = RotOf(angle);
    for (int i = 0; i < s.count; ++i) {
        s.verts[i] = Mul(xf, s.verts[i]);
        s.normals[i] = Mul(xf.q, s.normals[i]);
    }
}

// ComputeCentroid (Collision/Shapes/b2PolygonShape.cpp:77-117): triangle fan from the origin.
static Vec2 PolygonCentroid(const Vec2* vs, int count)
{
    Vec2 c = V(0.0f, 0.0f);
    float area = 0.0f;
    Vec2 pRef = V(0.0f, 0.0f);
    const float inv3 = 1.0f / 3.0f;
    for (int i = 0; i < count; ++i) {
        Vec2 p1 = pRef, p2 = vs[i], p3 = i + 1 < count ? vs[i + 1] : vs[0];
        Vec2 e1 = p2 - p1, e2 = p3 - p1;
        float D = Cross(e1, e2);
        float triangleArea = 0.5f * D;
        area += triangleArea;
        c = c + (triangleArea * inv3) * (p1 + p2 + p3);
    }
    float inv = 1.0f / area;
    c.x *= inv;
    c.y *= inv;
    return c;
}

// b2PolygonShape::Set (Collision/Shapes/b2PolygonShape.cpp:119-252): weld, gift-wrap hull, normals.
void PolygonSet(Shape& s, const Vec2* vertices, int count)
{
    if (count < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    int n = Min(count, kMaxPolygonVertices);
    Vec2 ps[kMaxPolygonVertices];
    int tempCount = 0;
    for (int i = 0; i < n; ++i) {
        Vec2 v = vertices[i];
        bool unique = true;
        for (int j = 0; j < tempCount; ++j) {
            if (DistanceSq(v, ps[j]) < 0.5f * kLinearSlop) { unique = false; break; }
        }
        if (unique) ps[tempCount++] = v;
    }
    n = tempCount;
    if (n < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    int i0 = 0;
    float x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        float x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
    }
    int hull[kMaxPolygonVertices];
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
        if (ie == i0) break;
    }
    if (m < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return; }
    s.type = kPolygon;
    s.radius = kPolygonRadius;
    s.count = m;
    for (int i = 0; i < m; ++i) s.verts[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        int i2 = i + 1 < m ? i + 1 : 0;
        Vec2 edge = s.verts[i2] - s.verts[i];
        s.normals[i] = Cross(edge, 1.0f);
        Normalize(s.normals[i]);
    }
    s.centroid = PolygonCentroid(s.verts, m);
}

// ComputeMass: polygon (b2PolygonShape.cpp:361-437), circle (b2CircleShape.cpp:95-101), edge (b2EdgeShape.cpp:132-138)
void ComputeMass(const Shape& s, float density, MassData* md)
{
    if (s.type == kCircle) {
        md->mass = density * kPi * s.radius * s.radius;
        md->center = s.p;
        md->I = md->mass * (0.5f * s.radius * s.radius + Dot(s.p, s.p));
        return;
    }
    if (s.type == kEdge) {
        md->mass = 0.0f;
        md->center = 0.5f * (s.v1 + s.v2);
        md->I = 0.0f;
        return;
    }
    Vec2 center = V(0.0f, 0.0f);
    float area = 0.0f, I = 0.0f;
    Vec2 ref = V(0.0f, 0.0f);
    for (int i = 0; i < s.count; ++i) ref = ref + s.verts[i];
    float invCount = 1.0f / s.count;
    ref.x *= invCount;
    ref.y *= invCount;
    const float k_inv3 = 1.0f / 3.0f;
    for (int i = 0; i < s.count; ++i) {
        Vec2 e1 = s.verts[i] - ref;
        Vec2 e2 = i + 1 < s.count ? s.verts[i + 1] - ref : s.verts[0] - ref;
        float D = Cross(e1, e2);
        float triangleArea = 0.5f * D;
        area += triangleArea;
        center = center + (triangleArea * k_inv3) * (e1 + e2);
        float ex1 = e1.x, ey1 = e1.y, ex2 = e2.x, ey2 = e2.y;
        float intx2 = ex1 * ex1 + ex2 * ex1 + ex2 * ex2;
        float inty2 = ey1 * ey1 + ey2 * ey1 + ey2 * ey2;
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
// a chain's child edge without the radius (b2ChainShape.cpp:171-187)
void ComputeAABB(const Shape& s, const Xf& xf, AABB* out)
{
    if (s.type == kCircle) {
        Vec2 p = xf.p + Mul(xf.q, s.p);
        out->lo = V(p.x - s.radius, p.y - s.radius);
        out->hi = V(p.x + s.radius, p.y + s.radius);
        return;
    }
    Vec2 lower, upper;
    if (s.type == kEdge) {
        Vec2 a = Mul(xf, s.v1), b = Mul(xf, s.v2);
        lower = Min(a, b);
        upper = Max(a, b);
        if (s.chain) {
            out->lo = lower;
            out->hi = upper;
            return;
        }
    } else {
        lower = Mul(xf, s.verts[0]);
        upper = lower;
        for (int i = 1; i < s.count; ++i) {
            Vec2 v = Mul(xf, s.verts[i]);
            lower = Min(lower, v);
            upper = Max(upper, v);
        }
    }
    Vec2 r = V(s.radius, s.radius);
    out->lo = lower - r;
    out->hi = upper + r;
}

// ---------------------------------------------------------------- manifolds
// b2WorldManifold::Initialize (Collision/b2Collision.cpp:22-87)
void WorldManifoldInit(WorldManifold* wm, const Manifold* m, const Xf& xfA, float radiusA, const Xf& xfB, float radiusB)
{
    if (m->pointCount == 0) return;
    switch (m->type) {
    case kCircles: {
        wm->normal = V(1.0f, 0.0f);
        Vec2 pointA = Mul(xfA, m->localPoint);
        Vec2 pointB = Mul(xfB, m->points[0].localPoint);
        if (DistanceSq(pointA, pointB) > kEpsilon * kEpsilon) {
            wm->normal = pointB - pointA;
            Normalize(wm->normal);
        }
        Vec2 cA = pointA + radiusA * wm->normal;
        Vec2 cB = pointB - radiusB * wm->normal;
        wm->points[0] = 0.5f * (cA + cB);
        wm->separations[0] = Dot(cB - cA, wm->normal);
        break;
    }
    case kFaceA: {
        wm->normal = Mul(xfA.q, m->localNormal);
        Vec2 planePoint = Mul(xfA, m->localPoint);
        for (int i = 0; i < m->pointCount; ++i) {
            Vec2 clipPoint = Mul(xfB, m->points[i].localPoint);
            Vec2 cA = clipPoint + (radiusA - Dot(clipPoint - planePoint, wm->normal)) * wm->normal;
            Vec2 cB = clipPoint - radiusB * wm->normal;
            wm->points[i] = 0.5f * (cA + cB);
            wm->separations[i] = Dot(cB - cA, wm->normal);
        }
        break;
    }
    case kFaceB: {
        wm->normal = Mul(xfB.q, m->localNormal);
        Vec2 planePoint = Mul(xfB, m->localPoint);
        for (int i = 0; i < m->pointCount; ++i) {
            Vec2 clipPoint = Mul(xfA, m->points[i].localPoint);
            Vec2 cB = clipPoint + (radiusB - Dot(clipPoint - planePoint, wm->normal)) * wm->normal;
            Vec2 cA = clipPoint - radiusA * wm->normal;
            wm->points[i] = 0.5f * (cA + cB);
            wm->separations[i] = Dot(cA - cB, wm->normal);
        }
        wm->normal = -wm->normal;
        break;
    }
    }
}

struct ClipVertex { Vec2 v; uint32_t id; };

// b2ClipSegmentToLine (Collision/b2Collision.cpp:204-235)
static int ClipSegmentToLine(ClipVertex vOut[2], const ClipVertex vIn[2], Vec2 normal, float offset, int vertexIndexA)
{
    int numOut = 0;
    float distance0 = Dot(normal, vIn[0].v) - offset;
    float distance1 = Dot(normal, vIn[1].v) - offset;
    if (distance0 <= 0.0f) vOut[numOut++] = vIn[0];
    if (distance1 <= 0.0f) vOut[numOut++] = vIn[1];
    if (distance0 * distance1 < 0.0f) {
        float interp = distance0 / (distance0 - distance1);
        vOut[numOut].v = vIn[0].v + interp * (vIn[1].v - vIn[0].v);
        vOut[numOut].id = MakeId(vertexIndexA, IdIndexB(vIn[0].id), kFeatureVertex, kFeatureFace);
        ++numOut;
    }
    return numOut;
}

// b2CollideCircles (Collision/b2CollideCircle.cpp:25-51)
void CollideCircles(Manifold* m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB)
{
    m->pointCount = 0;
    Vec2 pA = Mul(xfA, a.p), pB = Mul(xfB, b.p);
    Vec2 d = pB - pA;
    float distSqr = Dot(d, d);
    float radius = a.radius + b.radius;
    if (distSqr > radius * radius) return;
    m->type = kCircles;
    m->localPoint = a.p;
    m->localNormal = V(0.0f, 0.0f);
    m->pointCount = 1;
    m->points[0].localPoint = b.p;
    m->points[0].id = 0;
}

// b2CollidePolygonAndCircle (Collision/b2CollideCircle.cpp:53-154)
void CollidePolygonAndCircle(Manifold* m, const Shape& poly, const Xf& xfA, const Shape& circ, const Xf& xfB)
{
    m->pointCount = 0;
    Vec2 c = Mul(xfB, circ.p);
    Vec2 cLocal = MulT(xfA, c);
    int normalIndex = 0;
    float separation = -kMaxFloat;
    float radius = poly.radius + circ.radius;
    int vertexCount = poly.count;
    for (int i = 0; i < vertexCount; ++i) {
        float s = Dot(poly.normals[i], cLocal - poly.verts[i]);
        if (s > radius) return;
        if (s > separation) { separation = s; normalIndex = i; }
    }
    int vi1 = normalIndex, vi2 = vi1 + 1 < vertexCount ? vi1 + 1 : 0;
    Vec2 v1 = poly.verts[vi1], v2 = poly.verts[vi2];
    if (separation < kEpsilon) {
        m->pointCount = 1;
        m->type = kFaceA;
        m->localNormal = poly.normals[normalIndex];
        m->localPoint = 0.5f * (v1 + v2);
        m->points[0].localPoint = circ.p;
        m->points[0].id = 0;
        return;
    }
    float u1 = Dot(cLocal - v1, v2 - v1);
    float u2 = Dot(cLocal - v2, v1 - v2);
    if (u1 <= 0.0f) {
        if (DistanceSq(cLocal, v1) > radius * radius) return;
        m->pointCount = 1;
        m->type = kFaceA;
        m->localNormal = cLocal - v1;
        Normalize(m->localNormal);
        m->localPoint = v1;
        m->points[0].localPoint = circ.p;
        m->points[0].id = 0;
    } else if (u2 <= 0.0f) {
        if (DistanceSq(cLocal, v2) > radius * radius) return;
        m->pointCount = 1;
        m->type = kFaceA;
        m->localNormal = cLocal - v2;
        Normalize(m->localNormal);
        m->localPoint = v2;
        m->points[0].localPoint = circ.p;
        m->points[0].id = 0;
    } else {
        Vec2 faceCenter = 0.5f * (v1 + v2);
        float sep = Dot(cLocal - faceCenter, poly.normals[vi1]);
        if (sep > radius) return;
        m->pointCount = 1;
        m->type = kFaceA;
        m->localNormal = poly.normals[vi1];
        m->localPoint = faceCenter;
        m->points[0].localPoint = circ.p;
        m->points[0].id = 0;
    }
}

// b2FindMaxSeparation (Collision/b2CollidePolygon.cpp:28-67)
static float FindMaxSeparation(int* edgeIndex, const Shape& p1, const Xf& xf1, const Shape& p2, const Xf& xf2)
{
    Xf xf = MulT(xf2, xf1);
    int bestIndex = 0;
    float maxSeparation = -kMaxFloat;
    for (int i = 0; i < p1.count; ++i) {
        Vec2 n = Mul(xf.q, p1.normals[i]);
        Vec2 v1 = Mul(xf, p1.verts[i]);
        float si = kMaxFloat;
        for (int j = 0; j < p2.count; ++j) {
            float sij = Dot(n, p2.verts[j] - v1);
            if (sij < si) si = sij;
        }
        if (si > maxSeparation) { maxSeparation = si; bestIndex = i; }
    }
    *edgeIndex = bestIndex;
    return maxSeparation;
}

// b2FindIncidentEdge (Collision/b2CollidePolygon.cpp:69-110)
static void FindIncidentEdge(ClipVertex c[2], const Shape& p1, const Xf& xf1, int edge1, const Shape& p2, const Xf& xf2)
{
    Vec2 normal1 = MulT(xf2.q, Mul(xf1.q, p1.normals[edge1]));
    int index = 0;
    float minDot = kMaxFloat;
    for (int i = 0; i < p2.count; ++i) {
        float dot = Dot(normal1, p2.normals[i]);
        if (dot < minDot) { minDot = dot; index = i; }
    }
    int i1 = index, i2 = i1 + 1 < p2.count ? i1 + 1 : 0;
    c[0].v = Mul(xf2, p2.verts[i1]);
    c[0].id = MakeId(edge1, i1, kFeatureFace, kFeatureVertex);
    c[1].v = Mul(xf2, p2.verts[i2]);
    c[1].id = MakeId(edge1, i2, kFeatureFace, kFeatureVertex);
}

// b2CollidePolygons (Collision/b2CollidePolygon.cpp:121-239)
void CollidePolygons(Manifold* m, const Shape& polyA, const Xf& xfA, const Shape& polyB, const Xf& xfB)
{
    m->pointCount = 0;
    float totalRadius = polyA.radius + polyB.radius;
    int edgeA = 0;
    float separationA = FindMaxSeparation(&edgeA, polyA, xfA, polyB, xfB);
    if (separationA > totalRadius) return;
    int edgeB = 0;
    float separationB = FindMaxSeparation(&edgeB, polyB, xfB, polyA, xfA);
    if (separationB > totalRadius) return;
    const Shape *poly1, *poly2;
    Xf xf1, xf2;
    int edge1;
    bool flip;
    const float k_tol = 0.1f * kLinearSlop;
    if (separationB > separationA + k_tol) {
        poly1 = &polyB; poly2 = &polyA; xf1 = xfB; xf2 = xfA; edge1 = edgeB;
        m->type = kFaceB;
        flip = true;
    } else {
        poly1 = &polyA; poly2 = &polyB; xf1 = xfA; xf2 = xfB; edge1 = edgeA;
        m->type = kFaceA;
        flip = false;
    }
    ClipVertex incidentEdge[2];
    FindIncidentEdge(incidentEdge, *poly1, xf1, edge1, *poly2, xf2);
    int count1 = poly1->count;
    int iv1 = edge1, iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
    Vec2 v11 = poly1->verts[iv1], v12 = poly1->verts[iv2];
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
    ClipVertex clip1[2], clip2[2];
    if (ClipSegmentToLine(clip1, incidentEdge, -tangent, sideOffset1, iv1) < 2) return;
    if (ClipSegmentToLine(clip2, clip1, tangent, sideOffset2, iv2) < 2) return;
    m->localNormal = localNormal;
    m->localPoint = planePoint;
    int pointCount = 0;
    for (int i = 0; i < kMaxManifoldPoints; ++i) {
        float separation = Dot(normal, clip2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            ManifoldPoint* cp = m->points + pointCount;
            cp->localPoint = MulT(xf2, clip2[i].v);
            cp->id = flip ? IdFlip(clip2[i].id) : clip2[i].id;
            ++pointCount;
        }
    }
    m->pointCount = pointCount;
}

// b2CollideEdgeAndCircle (Collision/b2CollideEdge.cpp:29-147)
void CollideEdgeAndCircle(Manifold* m, const Shape& edge, const Xf& xfA, const Shape& circ, const Xf& xfB)
{
    m->pointCount = 0;
    Vec2 Q = MulT(xfA, Mul(xfB, circ.p));
    Vec2 A = edge.v1, B = edge.v2;
    Vec2 e = B - A;
    float u = Dot(e, B - Q);
    float v = Dot(e, Q - A);
    float radius = edge.radius + circ.radius;
    if (v <= 0.0f) {
        Vec2 d = Q - A;
        if (Dot(d, d) > radius * radius) return;
        if (edge.hasV0) {
            Vec2 e1 = A - edge.v0;
            float u1 = Dot(e1, A - Q);
            if (u1 > 0.0f) return;
        }
        m->pointCount = 1;
        m->type = kCircles;
        m->localNormal = V(0.0f, 0.0f);
        m->localPoint = A;
        m->points[0].id = MakeId(0, 0, kFeatureVertex, kFeatureVertex);
        m->points[0].localPoint = circ.p;
        return;
    }
    if (u <= 0.0f) {
        Vec2 d = Q - B;
        if (Dot(d, d) > radius * radius) return;
        if (edge.hasV3) {
            Vec2 e2 = edge.v3 - B;
            float v2 = Dot(e2, Q - B);
            if (v2 > 0.0f) return;
        }
        m->pointCount = 1;
        m->type = kCircles;
        m->localNormal = V(0.0f, 0.0f);
        m->localPoint = B;
        m->points[0].id = MakeId(1, 0, kFeatureVertex, kFeatureVertex);
        m->points[0].localPoint = circ.p;
        return;
    }
    float den = Dot(e, e);
    Vec2 P = (1.0f / den) * (u * A + v * B);
    Vec2 d = Q - P;
    if (Dot(d, d) > radius * radius) return;
    Vec2 n = V(-e.y, e.x);
    if (Dot(n, Q - A) < 0.0f) n = V(-n.x, -n.y);
    Normalize(n);
    m->pointCount = 1;
    m->type = kFaceA;
    m->localNormal = n;
    m->localPoint = A;
    m->points[0].id = MakeId(0, 0, kFeatureFace, kFeatureVertex);
    m->points[0].localPoint = circ.p;
}

// b2EPCollider (Collision/b2CollideEdge.cpp:149-692): edge versus polygon with edge adjacency.
namespace {
enum AxisType { kAxisUnknown = 0, kAxisEdgeA, kAxisEdgeB };
struct EPAxis { int type; int index; float separation; };
struct EPState {
    Vec2 pv[kMaxPolygonVertices], pn[kMaxPolygonVertices];
    int count;
    Xf xf;
    Vec2 centroidB, v0, v1, v2, v3, normal0, normal1, normal2, normal, lowerLimit, upperLimit;
    float radius;
    bool front;
};

EPAxis EdgeSeparation(const EPState& s)
{
    EPAxis axis;
    axis.type = kAxisEdgeA;
    axis.index = s.front ? 0 : 1;
    axis.separation = FLT_MAX;
    for (int i = 0; i < s.count; ++i) {
        float sep = Dot(s.normal, s.pv[i] - s.v1);
        if (sep < axis.separation) axis.separation = sep;
    }
    return axis;
}

EPAxis PolygonSeparation(const EPState& s)
{
    EPAxis axis;
    axis.type = kAxisUnknown;
    axis.index = -1;
    axis.separation = -FLT_MAX;
    Vec2 perp = V(-s.normal.y, s.normal.x);
    for (int i = 0; i < s.count; ++i) {
        Vec2 n = -s.pn[i];
        float s1 = Dot(n, s.pv[i] - s.v1);
        float s2 = Dot(n, s.pv[i] - s.v2);
        float sep = Min(s1, s2);
        if (sep > s.radius) {
            axis.type = kAxisEdgeB;
            axis.index = i;
            axis.separation = sep;
            return axis;
        }
        if (Dot(n, perp) >= 0.0f) {
            if (Dot(n - s.upperLimit, s.normal) < -kAngularSlop) continue;
        } else {
            if (Dot(n - s.lowerLimit, s.normal) < -kAngularSlop) continue;
        }
        if (sep > axis.separation) {
            axis.type = kAxisEdgeB;
            axis.index = i;
            axis.separation = sep;
        }
    }
    return axis;
}
} // namespace

void CollideEdgeAndPolygon(Manifold* m, const Shape& edge, const Xf& xfA, const Shape& poly, const Xf& xfB)
{
    EPState s;
    s.normal0 = V(0.0f, 0.0f);
    s.normal2 = V(0.0f, 0.0f);
    s.xf = MulT(xfA, xfB);
    s.centroidB = Mul(s.xf, poly.centroid);
    s.v0 = edge.v0; s.v1 = edge.v1; s.v2 = edge.v2; s.v3 = edge.v3;
    bool hasVertex0 = edge.hasV0, hasVertex3 = edge.hasV3;
    Vec2 edge1 = s.v2 - s.v1;
    Normalize(edge1);
    s.normal1 = V(edge1.y, -edge1.x);
    float offset1 = Dot(s.normal1, s.centroidB - s.v1);
    float offset0 = 0.0f, offset2 = 0.0f;
    bool convex1 = false, convex2 = false;
    if (hasVertex0) {
        Vec2 edge0 = s.v1 - s.v0;
        Normalize(edge0);
        s.normal0 = V(edge0.y, -edge0.x);
        convex1 = Cross(edge0, edge1) >= 0.0f;
        offset0 = Dot(s.normal0, s.centroidB - s.v0);
    }
    if (hasVertex3) {
        Vec2 edge2 = s.v3 - s.v2;
        Normalize(edge2);
        s.normal2 = V(edge2.y, -edge2.x);
        convex2 = Cross(edge1, edge2) > 0.0f;
        offset2 = Dot(s.normal2, s.centroidB - s.v2);
    }
    const Vec2 n0 = s.normal0, n1 = s.normal1, n2 = s.normal2;
    // Front/back classification and normal limits (b2CollideEdge.cpp:287-433).
    if (hasVertex0 && hasVertex3) {
        if (convex1 && convex2) {
            s.front = offset0 >= 0.0f || offset1 >= 0.0f || offset2 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = n0; s.upperLimit = n2; }
            else { s.normal = -n1; s.lowerLimit = -n1; s.upperLimit = -n1; }
        } else if (convex1) {
            s.front = offset0 >= 0.0f || (offset1 >= 0.0f && offset2 >= 0.0f);
            if (s.front) { s.normal = n1; s.lowerLimit = n0; s.upperLimit = n1; }
            else { s.normal = -n1; s.lowerLimit = -n2; s.upperLimit = -n1; }
        } else if (convex2) {
            s.front = offset2 >= 0.0f || (offset0 >= 0.0f && offset1 >= 0.0f);
            if (s.front) { s.normal = n1; s.lowerLimit = n1; s.upperLimit = n2; }
            else { s.normal = -n1; s.lowerLimit = -n1; s.upperLimit = -n0; }
        } else {
            s.front = offset0 >= 0.0f && offset1 >= 0.0f && offset2 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = n1; s.upperLimit = n1; }
            else { s.normal = -n1; s.lowerLimit = -n2; s.upperLimit = -n0; }
        }
    } else if (hasVertex0) {
        if (convex1) {
            s.front = offset0 >= 0.0f || offset1 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = n0; s.upperLimit = -n1; }
            else { s.normal = -n1; s.lowerLimit = n1; s.upperLimit = -n1; }
        } else {
            s.front = offset0 >= 0.0f && offset1 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = n1; s.upperLimit = -n1; }
            else { s.normal = -n1; s.lowerLimit = n1; s.upperLimit = -n0; }
        }
    } else if (hasVertex3) {
        if (convex2) {
            s.front = offset1 >= 0.0f || offset2 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = -n1; s.upperLimit = n2; }
            else { s.normal = -n1; s.lowerLimit = -n1; s.upperLimit = n1; }
        } else {
            s.front = offset1 >= 0.0f && offset2 >= 0.0f;
            if (s.front) { s.normal = n1; s.lowerLimit = -n1; s.upperLimit = n1; }
            else { s.normal = -n1; s.lowerLimit = -n2; s.upperLimit = n1; }
        }
    } else {
        s.front = offset1 >= 0.0f;
        if (s.front) { s.normal = n1; s.lowerLimit = -n1; s.upperLimit = -n1; }
        else { s.normal = -n1; s.lowerLimit = n1; s.upperLimit = n1; }
    }
    s.count = poly.count;
    for (int i = 0; i < poly.count; ++i) {
        s.pv[i] = Mul(s.xf, poly.verts[i]);
        s.pn[i] = Mul(s.xf.q, poly.normals[i]);
    }
    s.radius = 2.0f * kPolygonRadius;
    m->pointCount = 0;
    EPAxis edgeAxis = EdgeSeparation(s);
    if (edgeAxis.type == kAxisUnknown) return;
    if (edgeAxis.separation > s.radius) return;
    EPAxis polygonAxis = PolygonSeparation(s);
    if (polygonAxis.type != kAxisUnknown && polygonAxis.separation > s.radius) return;
    const float k_relativeTol = 0.98f, k_absoluteTol = 0.001f;
    EPAxis primary;
    if (polygonAxis.type == kAxisUnknown) primary = edgeAxis;
    else if (polygonAxis.separation > k_relativeTol * edgeAxis.separation + k_absoluteTol) primary = polygonAxis;
    else primary = edgeAxis;

    ClipVertex ie[2];
    int rfI1, rfI2;
    Vec2 rfV1, rfV2, rfNormal;
    if (primary.type == kAxisEdgeA) {
        m->type = kFaceA;
        int bestIndex = 0;
        float bestValue = Dot(s.normal, s.pn[0]);
        for (int i = 1; i < s.count; ++i) {
            float value = Dot(s.normal, s.pn[i]);
            if (value < bestValue) { bestValue = value; bestIndex = i; }
        }
        int i1 = bestIndex, i2 = i1 + 1 < s.count ? i1 + 1 : 0;
        ie[0].v = s.pv[i1];
        ie[0].id = MakeId(0, i1, kFeatureFace, kFeatureVertex);
        ie[1].v = s.pv[i2];
        ie[1].id = MakeId(0, i2, kFeatureFace, kFeatureVertex);
        if (s.front) { rfI1 = 0; rfI2 = 1; rfV1 = s.v1; rfV2 = s.v2; rfNormal = s.normal1; }
        else { rfI1 = 1; rfI2 = 0; rfV1 = s.v2; rfV2 = s.v1; rfNormal = -s.normal1; }
    } else {
        m->type = kFaceB;
        ie[0].v = s.v1;
        ie[0].id = MakeId(0, primary.index, kFeatureVertex, kFeatureFace);
        ie[1].v = s.v2;
        ie[1].id = MakeId(0, primary.index, kFeatureVertex, kFeatureFace);
        rfI1 = primary.index;
        rfI2 = rfI1 + 1 < s.count ? rfI1 + 1 : 0;
        rfV1 = s.pv[rfI1];
        rfV2 = s.pv[rfI2];
        rfNormal = s.pn[rfI1];
    }
    Vec2 sideNormal1 = V(rfNormal.y, -rfNormal.x);
    Vec2 sideNormal2 = -sideNormal1;
    float sideOffset1 = Dot(sideNormal1, rfV1);
    float sideOffset2 = Dot(sideNormal2, rfV2);
    ClipVertex clip1[2], clip2[2];
    if (ClipSegmentToLine(clip1, ie, sideNormal1, sideOffset1, rfI1) < kMaxManifoldPoints) return;
    if (ClipSegmentToLine(clip2, clip1, sideNormal2, sideOffset2, rfI2) < kMaxManifoldPoints) return;
    if (primary.type == kAxisEdgeA) {
        m->localNormal = rfNormal;
        m->localPoint = rfV1;
    } else {
        m->localNormal = poly.normals[rfI1];
        m->localPoint = poly.verts[rfI1];
    }
    int pointCount = 0;
    for (int i = 0; i < kMaxManifoldPoints; ++i) {
        float separation = Dot(rfNormal, clip2[i].v - rfV1);
        if (separation <= s.radius) {
            ManifoldPoint* cp = m->points + pointCount;
            if (primary.type == kAxisEdgeA) {
                cp->localPoint = MulT(s.xf, clip2[i].v);
                cp->id = clip2[i].id;
            } else {
                cp->localPoint = clip2[i].v;
                cp->id = IdFlip(clip2[i].id);
            }
            ++pointCount;
        }
    }
    m->pointCount = pointCount;
}

// ---------------------------------------------------------------- distance (GJK)
// b2DistanceProxy::Set (Collision/b2Distance.cpp:28-78) for circle, polygon and edge.
void ProxyOf(DistanceProxy* p, const Shape& s)
{
    if (s.type == kCircle) { p->verts = &s.p; p->count = 1; }
    else if (s.type == kEdge) { p->verts = &s.v1; p->count = 2; }
    else { p->verts = s.verts; p->count = s.count; }
    p->radius = s.radius;
}

static int Support(const DistanceProxy& p, Vec2 d)
{
    int best = 0;
    float bestValue = Dot(p.verts[0], d);
    for (int i = 1; i < p.count; ++i) {
        float value = Dot(p.verts[i], d);
        if (value > bestValue) { best = i; bestValue = value; }
    }
    return best;
}

namespace {
struct SimplexVertex { Vec2 wA, wB, w; float a; int indexA, indexB; };
struct Simplex {
    SimplexVertex v[3];
    int count;

    float Metric() const
    {
        switch (count) {
        case 2: return Distance(v[0].w, v[1].w);
        case 3: return Cross(v[1].w - v[0].w, v[2].w - v[0].w);
        default: return 0.0f;
        }
    }
    // b2Simplex::ReadCache (Collision/b2Distance.cpp:94-141)
    void ReadCache(const SimplexCache* cache, const DistanceProxy& pa, const Xf& xfA, const DistanceProxy& pb, const Xf& xfB)
    {
        count = cache->count;
        for (int i = 0; i < count; ++i) {
            SimplexVertex* sv = v + i;
            sv->indexA = cache->indexA[i];
            sv->indexB = cache->indexB[i];
            sv->wA = Mul(xfA, pa.verts[sv->indexA]);
            sv->wB = Mul(xfB, pb.verts[sv->indexB]);
            sv->w = sv->wB - sv->wA;
            sv->a = 0.0f;
        }
        if (count > 1) {
            float metric1 = cache->metric, metric2 = Metric();
            if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < kEpsilon) count = 0;
        }
        if (count == 0) {
            SimplexVertex* sv = v;
            sv->indexA = 0;
            sv->indexB = 0;
            sv->wA = Mul(xfA, pa.verts[0]);
            sv->wB = Mul(xfB, pb.verts[0]);
            sv->w = sv->wB - sv->wA;
            sv->a = 1.0f;
            count = 1;
        }
    }
    void WriteCache(SimplexCache* cache) const
    {
        cache->metric = Metric();
        cache->count = count;
        for (int i = 0; i < count; ++i) {
            cache->indexA[i] = (uint8_t)v[i].indexA;
            cache->indexB[i] = (uint8_t)v[i].indexB;
        }
    }
    Vec2 SearchDirection() const
    {
        if (count == 1) return -v[0].w;
        Vec2 e12 = v[1].w - v[0].w;
        float sgn = Cross(e12, -v[0].w);
        if (sgn > 0.0f) return Cross(1.0f, e12);
        return Cross(e12, 1.0f);
    }
    Vec2 ClosestPoint() const
    {
        if (count == 1) return v[0].w;
        if (count == 2) return v[0].a * v[0].w + v[1].a * v[1].w;
        return V(0.0f, 0.0f);
    }
    void Witness(Vec2* pA, Vec2* pB) const
    {
        if (count == 1) { *pA = v[0].wA; *pB = v[0].wB; }
        else if (count == 2) {
            *pA = v[0].a * v[0].wA + v[1].a * v[1].wA;
            *pB = v[0].a * v[0].wB + v[1].a * v[1].wB;
        } else {
            *pA = v[0].a * v[0].wA + v[1].a * v[1].wA + v[2].a * v[2].wA;
            *pB = *pA;
        }
    }
    // b2Simplex::Solve2 (Collision/b2Distance.cpp:255-283)
    void Solve2()
    {
        Vec2 w1 = v[0].w, w2 = v[1].w;
        Vec2 e12 = w2 - w1;
        float d12_2 = -Dot(w1, e12);
        if (d12_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        float d12_1 = Dot(w2, e12);
        if (d12_1 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        float inv = 1.0f / (d12_1 + d12_2);
        v[0].a = d12_1 * inv;
        v[1].a = d12_2 * inv;
        count = 2;
    }
    // b2Simplex::Solve3 (Collision/b2Distance.cpp:296-400)
    void Solve3()
    {
        Vec2 w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
        Vec2 e12 = w2 - w1;
        float w1e12 = Dot(w1, e12), w2e12 = Dot(w2, e12);
        float d12_1 = w2e12, d12_2 = -w1e12;
        Vec2 e13 = w3 - w1;
        float w1e13 = Dot(w1, e13), w3e13 = Dot(w3, e13);
        float d13_1 = w3e13, d13_2 = -w1e13;
        Vec2 e23 = w3 - w2;
        float w2e23 = Dot(w2, e23), w3e23 = Dot(w3, e23);
        float d23_1 = w3e23, d23_2 = -w2e23;
        float n123 = Cross(e12, e13);
        float d123_1 = n123 * Cross(w2, w3);
        float d123_2 = n123 * Cross(w3, w1);
        float d123_3 = n123 * Cross(w1, w2);
        if (d12_2 <= 0.0f && d13_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
            float inv = 1.0f / (d12_1 + d12_2);
            v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; count = 2; return;
        }
        if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
            float inv = 1.0f / (d13_1 + d13_2);
            v[0].a = d13_1 * inv; v[2].a = d13_2 * inv; count = 2; v[1] = v[2]; return;
        }
        if (d12_1 <= 0.0f && d23_2 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        if (d13_1 <= 0.0f && d23_1 <= 0.0f) { v[2].a = 1.0f; count = 1; v[0] = v[2]; return; }
        if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
            float inv = 1.0f / (d23_1 + d23_2);
            v[1].a = d23_1 * inv; v[2].a = d23_2 * inv; count = 2; v[0] = v[2]; return;
        }
        float inv = 1.0f / (d123_1 + d123_2 + d123_3);
        v[0].a = d123_1 * inv; v[1].a = d123_2 * inv; v[2].a = d123_3 * inv; count = 3;
    }
};
} // namespace

// b2Distance (Collision/b2Distance.cpp:402-535)
void Distance(DistanceOutput* out, SimplexCache* cache, const DistanceProxy& pa, const Xf& xfA,
              const DistanceProxy& pb, const Xf& xfB, bool useRadii)
{
    Simplex simplex;
    simplex.ReadCache(cache, pa, xfA, pb, xfB);
    const int k_maxIters = 20;
    int saveA[3], saveB[3];
    int iter = 0;
    while (iter < k_maxIters) {
        int saveCount = simplex.count;
        for (int i = 0; i < saveCount; ++i) { saveA[i] = simplex.v[i].indexA; saveB[i] = simplex.v[i].indexB; }
        if (simplex.count == 2) simplex.Solve2();
        else if (simplex.count == 3) simplex.Solve3();
        if (simplex.count == 3) break;
        Vec2 d = simplex.SearchDirection();
        if (LengthSq(d) < kEpsilon * kEpsilon) break;
        SimplexVertex* vertex = simplex.v + simplex.count;
        vertex->indexA = Support(pa, MulT(xfA.q, -d));
        vertex->wA = Mul(xfA, pa.verts[vertex->indexA]);
        vertex->indexB = Support(pb, MulT(xfB.q, d));
        vertex->wB = Mul(xfB, pb.verts[vertex->indexB]);
        vertex->w = vertex->wB - vertex->wA;
        ++iter;
        bool duplicate = false;
        for (int i = 0; i < saveCount; ++i) {
            if (vertex->indexA == saveA[i] && vertex->indexB == saveB[i]) { duplicate = true; break; }
        }
        if (duplicate) break;
        ++simplex.count;
    }
    simplex.Witness(&out->pointA, &out->pointB);
    out->distance = Distance(out->pointA, out->pointB);
    out->iterations = iter;
    simplex.WriteCache(cache);
    if (useRadii) {
        float rA = pa.radius, rB = pb.radius;
        if (out->distance > rA + rB && out->distance > kEpsilon) {
            out->distance -= rA + rB;
            Vec2 normal = out->pointB - out->pointA;
            Normalize(normal);
            out->pointA = out->pointA + rA * normal;
            out->pointB = out->pointB - rB * normal;
        } else {
            Vec2 p = 0.5f * (out->pointA + out->pointB);
            out->pointA = p;
            out->pointB = p;
            out->distance = 0.0f;
        }
    }
}

// ---------------------------------------------------------------- time of impact
namespace {
enum SepType { kSepPoints = 0, kSepFaceA, kSepFaceB };
// b2SeparationFunction (Collision/b2TimeOfImpact.cpp:33-240)
struct SepFn {
    const DistanceProxy *pa, *pb;
    Sweep sa, sb;
    int type;
    Vec2 localPoint, axis;

    float Init(const SimplexCache* cache, const DistanceProxy& A, const Sweep& swA, const DistanceProxy& B, const Sweep& swB, float t1)
    {
        pa = &A; pb = &B;
        int count = cache->count;
        sa = swA; sb = swB;
        Xf xfA, xfB;
        SweepXf(sa, &xfA, t1);
        SweepXf(sb, &xfB, t1);
        if (count == 1) {
            type = kSepPoints;
            Vec2 pointA = Mul(xfA, pa->verts[cache->indexA[0]]);
            Vec2 pointB = Mul(xfB, pb->verts[cache->indexB[0]]);
            axis = pointB - pointA;
            return Normalize(axis);
        } else if (cache->indexA[0] == cache->indexA[1]) {
            type = kSepFaceB;
            Vec2 b1 = pb->verts[cache->indexB[0]], b2 = pb->verts[cache->indexB[1]];
            axis = Cross(b2 - b1, 1.0f);
            Normalize(axis);
            Vec2 normal = Mul(xfB.q, axis);
            localPoint = 0.5f * (b1 + b2);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 pointA = Mul(xfA, pa->verts[cache->indexA[0]]);
            float s = Dot(pointA - pointB, normal);
            if (s < 0.0f) { axis = -axis; s = -s; }
            return s;
        } else {
            type = kSepFaceA;
            Vec2 a1 = pa->verts[cache->indexA[0]], a2 = pa->verts[cache->indexA[1]];
            axis = Cross(a2 - a1, 1.0f);
            Normalize(axis);
            Vec2 normal = Mul(xfA.q, axis);
            localPoint = 0.5f * (a1 + a2);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 pointB = Mul(xfB, pb->verts[cache->indexB[0]]);
            float s = Dot(pointB - pointA, normal);
            if (s < 0.0f) { axis = -axis; s = -s; }
            return s;
        }
    }
    float FindMin(int* iA, int* iB, float t) const
    {
        Xf xfA, xfB;
        SweepXf(sa, &xfA, t);
        SweepXf(sb, &xfB, t);
        if (type == kSepPoints) {
            Vec2 axisA = MulT(xfA.q, axis), axisB = MulT(xfB.q, -axis);
            *iA = Support(*pa, axisA);
            *iB = Support(*pb, axisB);
            Vec2 pointA = Mul(xfA, pa->verts[*iA]), pointB = Mul(xfB, pb->verts[*iB]);
            return Dot(pointB - pointA, axis);
        } else if (type == kSepFaceA) {
            Vec2 normal = Mul(xfA.q, axis);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 axisB = MulT(xfB.q, -normal);
            *iA = -1;
            *iB = Support(*pb, axisB);
            Vec2 pointB = Mul(xfB, pb->verts[*iB]);
            return Dot(pointB - pointA, normal);
        } else {
            Vec2 normal = Mul(xfB.q, axis);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 axisA = MulT(xfA.q, -normal);
            *iB = -1;
            *iA = Support(*pa, axisA);
            Vec2 pointA = Mul(xfA, pa->verts[*iA]);
            return Dot(pointA - pointB, normal);
        }
    }
    float Eval(int iA, int iB, float t) const
    {
        Xf xfA, xfB;
        SweepXf(sa, &xfA, t);
        SweepXf(sb, &xfB, t);
        if (type == kSepPoints) {
            Vec2 pointA = Mul(xfA, pa->verts[iA]), pointB = Mul(xfB, pb->verts[iB]);
            return Dot(pointB - pointA, axis);
        } else if (type == kSepFaceA) {
            Vec2 normal = Mul(xfA.q, axis);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 pointB = Mul(xfB, pb->verts[iB]);
            return Dot(pointB - pointA, normal);
        } else {
            Vec2 normal = Mul(xfB.q, axis);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 pointA = Mul(xfA, pa->verts[iA]);
            return Dot(pointA - pointB, normal);
        }
    }
};
} // namespace

// b2TimeOfImpact (Collision/b2TimeOfImpact.cpp:257-481): conservative advancement.
void TimeOfImpact(int* state, float* tOut, const DistanceProxy& pa, const DistanceProxy& pb, const Sweep& swA0,
                  const Sweep& swB0, float tMax)
{
    *state = kToiUnknown;
    *tOut = tMax;
    Sweep sweepA = swA0, sweepB = swB0;
    SweepNormalize(sweepA);
    SweepNormalize(sweepB);
    float totalRadius = pa.radius + pb.radius;
    float target = Max(kLinearSlop, totalRadius - 3.0f * kLinearSlop);
    float tolerance = 0.25f * kLinearSlop;
    float t1 = 0.0f;
    const int k_maxIterations = 20;
    int iter = 0;
    SimplexCache cache;
    cache.count = 0;
    for (;;) {
        Xf xfA, xfB;
        SweepXf(sweepA, &xfA, t1);
        SweepXf(sweepB, &xfB, t1);
        DistanceOutput dout;
        Distance(&dout, &cache, pa, xfA, pb, xfB, false);
        if (dout.distance <= 0.0f) { *state = kToiOverlapped; *tOut = 0.0f; break; }
        if (dout.distance < target + tolerance) { *state = kToiTouching; *tOut = t1; break; }
        SepFn fcn;
        fcn.Init(&cache, pa, sweepA, pb, sweepB, t1);
        bool done = false;
        float t2 = tMax;
        int pushBackIter = 0;
        for (;;) {
            int indexA, indexB;
            float s2 = fcn.FindMin(&indexA, &indexB, t2);
            if (s2 > target + tolerance) { *state = kToiSeparated; *tOut = tMax; done = true; break; }
            if (s2 > target - tolerance) { t1 = t2; break; }
            float s1 = fcn.Eval(indexA, indexB, t1);
            if (s1 < target - tolerance) { *state = kToiFailed; *tOut = t1; done = true; break; }
            if (s1 <= target + tolerance) { *state = kToiTouching; *tOut = t1; done = true; break; }
            int rootIterCount = 0;
            float a1 = t1, a2 = t2;
            for (;;) {
                float t;
                if (rootIterCount & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5f * (a1 + a2);
                ++rootIterCount;
                float s = fcn.Eval(indexA, indexB, t);
                if (Abs(s - target) < tolerance) { t2 = t; break; }
                if (s > target) { a1 = t; s1 = s; }
                else { a2 = t; s2 = s; }
                if (rootIterCount == 50) break;
            }
            ++pushBackIter;
            if (pushBackIter == kMaxPolygonVertices) break;
        }
        ++iter;
        if (done) break;
        if (iter == k_maxIterations) { *state = kToiFailed; *tOut = t1; break; }
    }
}

} // namespace b2o
