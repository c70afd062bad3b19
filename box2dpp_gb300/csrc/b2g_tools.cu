// Element-wise device kernels exposed through the C-ABI for direct checks of the step's building
// blocks: the project sin/cos (b2Rot::Set, Box2D/Common/b2Math.h:305-312) and the narrowphase
// (b2Collide*, Box2D/Collision/b2Collision.h:170-200).
#include <cuda_runtime.h>

#include "b2g_core.h"

namespace b2g {

__global__ void SinCosKernel(const float* __restrict__ x, float* __restrict__ s, float* __restrict__ c, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float sv, cv;
        SinCos(x[i], &sv, &cv);
        s[i] = sv;
        c[i] = cv;
    }
}

__global__ void CollideKernel(int n, const Shape* a, const float4* xa, const Shape* b, const float4* xb, int4* oi, float4* of)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Xf A, B;
        A.p = V(xa[i].x, xa[i].y); A.q.s = xa[i].z; A.q.c = xa[i].w;
        B.p = V(xb[i].x, xb[i].y); B.q.s = xb[i].z; B.q.c = xb[i].w;
        Manifold m;
        m.count = 0;
        m.type = 0;
        m.localNormal = V(0.0f, 0.0f);
        m.localPoint = V(0.0f, 0.0f);
        Evaluate(&m, a[i], A, b[i], B);
        bool any = m.count > 0;
        oi[i] = make_int4(any ? m.type : 0, m.count, m.count > 0 ? (int)m.p[0].id : 0, m.count > 1 ? (int)m.p[1].id : 0);
        of[3 * i] = any ? make_float4(m.localNormal.x, m.localNormal.y, m.localPoint.x, m.localPoint.y)
                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        of[3 * i + 1] = m.count > 0 ? make_float4(m.p[0].lp.x, m.p[0].lp.y, 0.0f, 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        of[3 * i + 2] = m.count > 1 ? make_float4(m.p[1].lp.x, m.p[1].lp.y, 0.0f, 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

} // namespace b2g

cudaError_t b2gLaunchSinCos(const float* x, float* s, float* c, int n, cudaStream_t stream)
{
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    b2g::SinCosKernel<<<blocks, 256, 0, stream>>>(x, s, c, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

cudaError_t b2gLaunchCollide(int n, const b2g::Shape* a, const float4* xa, const b2g::Shape* b, const float4* xb,
                             int4* oi, float4* of, cudaStream_t stream)
{
    int blocks = (n + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    b2g::CollideKernel<<<blocks, 128, 0, stream>>>(n, a, xa, b, xb, oi, of);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

// ------------------------------------------------------------------ world queries
// b2World::QueryAABB and b2World::RayCast (Dynamics/b2World.cpp:965-1020) over one world of a batch,
// one thread per query.
#include "b2g_world.h"

namespace b2g {

// The fixtures whose broadphase fat AABB overlaps the query box (b2DynamicTree::Query reports every
// leaf whose box passes b2TestOverlap), in fixture order; fill == nullptr only counts them.
__global__ void QueryAabbKernel(Batch B, int w, const float4* boxes, int n, const int* offsets, int* counts,
                                int* fill, int cap)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const WorldDesc d = B.desc[w];
    const float4 q = boxes[i];
    int k = 0;
    for (int f = 0; f < d.fixCount; ++f) {
        const int proxy = B.fi[d.fixBase + f].z;
        if (proxy < 0) continue;
        if (!Overlap(B.fat[d.proxyBase + proxy], q)) continue;
        if (fill) {
            const int slot = offsets[i] + k;
            if (slot < cap) fill[slot] = f;
        }
        ++k;
    }
    if (!fill) counts[i] = k;
}

// The closest fixture hit by each segment p1 -> p2 (b2World::RayCast with a callback that clips the
// ray to every reported fraction): the smallest fraction over all fixtures, ties to the lowest
// fixture index; hit = fraction, point (1 - f) p1 + f p2, normal.
__global__ void RayCastKernel(Batch B, int w, const float4* rays, int n, int* fixture, float* hit)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const WorldDesc d = B.desc[w];
    const float4 r = rays[i];
    const Vec2 p1 = V(r.x, r.y), p2 = V(r.z, r.w);
    int best = -1;
    float bestF = 0.0f;
    Vec2 bestN = V(0.0f, 0.0f);
    for (int f = 0; f < d.fixCount; ++f) {
        // the tree holds only fixtures with a proxy (not those of inactive or destroyed bodies)
        const int4 fx = B.fi[d.fixBase + f];
        if (fx.z < 0 || fx.x < 0) continue;
        const int body = fx.x;
        const float4 x = B.xf[d.bodyBase + body];
        Xf xf;
        xf.p = V(x.x, x.y);
        xf.q.s = x.z;
        xf.q.c = x.w;
        float fr;
        Vec2 nrm;
        if (!RayCastShape(B.shape[d.fixBase + f], xf, p1, p2, 1.0f, &fr, &nrm)) continue;
        if (best < 0 || fr < bestF) { best = f; bestF = fr; bestN = nrm; }
    }
    fixture[i] = best;
    const Vec2 pt = best >= 0 ? (1.0f - bestF) * p1 + bestF * p2 : V(0.0f, 0.0f);
    hit[5 * i] = bestF;
    hit[5 * i + 1] = pt.x;
    hit[5 * i + 2] = pt.y;
    hit[5 * i + 3] = bestN.x;
    hit[5 * i + 4] = bestN.y;
}

// Every fixture the segment p1 -> p2 hits (b2Fixture::RayCast with maxFraction 1), one thread per
// fixture of the world: hits[k] = {fixture, fraction, normal.x, normal.y} appended at an atomic slot
// (order restored by the caller), *count the number of hits (slots past cap are not written).
__global__ void RayCastAllKernel(Batch B, int w, float4 ray, float4* hits, int* count, int cap)
{
    const WorldDesc d = B.desc[w];
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.fixCount) return;
    const int4 fx = B.fi[d.fixBase + f];
    if (fx.z < 0 || fx.x < 0) return;
    const float4 x = B.xf[d.bodyBase + fx.x];
    Xf xf;
    xf.p = V(x.x, x.y);
    xf.q.s = x.z;
    xf.q.c = x.w;
    float fr;
    Vec2 nrm;
    if (!RayCastShape(B.shape[d.fixBase + f], xf, V(ray.x, ray.y), V(ray.z, ray.w), 1.0f, &fr, &nrm)) return;
    const int slot = atomicAdd(count, 1);
    if (slot < cap) hits[slot] = make_float4(__int_as_float(f), fr, nrm.x, nrm.y);
}

} // namespace b2g

cudaError_t b2gLaunchRayCastAll(const b2g::Batch& B, int w, int fixCount, float4 ray, float4* hits, int* count, int cap,
                                cudaStream_t stream)
{
    if (fixCount <= 0) return cudaSuccess;
    b2g::RayCastAllKernel<<<(fixCount + 127) / 128, 128, 0, stream>>>(B, w, ray, hits, count, cap);
    return cudaGetLastError();
}

cudaError_t b2gLaunchQueryAabb(const b2g::Batch& B, int w, const float4* boxes, int n, const int* offsets, int* counts,
                               int* fill, int cap, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::QueryAabbKernel<<<(n + 127) / 128, 128, 0, stream>>>(B, w, boxes, n, offsets, counts, fill, cap);
    return cudaGetLastError();
}

cudaError_t b2gLaunchRayCast(const b2g::Batch& B, int w, const float4* rays, int n, int* fixture, float* hit,
                             cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    b2g::RayCastKernel<<<(n + 127) / 128, 128, 0, stream>>>(B, w, rays, n, fixture, hit);
    return cudaGetLastError();
}
