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
