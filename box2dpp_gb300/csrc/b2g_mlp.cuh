// The learned warm start's network: a BF16 MLP 14 -> 64 -> 64 -> 2 with ReLU, FP32 accumulation,
// evaluated on the tensor cores with mma.sync m16n8k16 (bf16 inputs, f32 accumulators). One warp
// evaluates a tile of 16 rows; the accumulator fragments of one layer are repacked in registers as
// the A fragments of the next, so hidden activations never leave the registers.
//
// Fragment layout of m16n8k16 (PTX ISA, mma .bf16): lane = 4 * g + t (g = lane >> 2, t = lane & 3).
//   A (16 x 16, row major): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..2t+1], a2 = A[g][2t+8..2t+9],
//                           a3 = A[g+8][2t+8..2t+9] (two bf16 per 32-bit register, lower column low)
//   B (16 x 8, column major): b0 = B[2t..2t+1][g], b1 = B[2t+8..2t+9][g]
//   C (16 x 8, f32): c0, c1 = C[g][2t..2t+1], c2, c3 = C[g+8][2t..2t+1]
// With weights stored as W[out][in] (row major), B[k][n] = W[n][k], so b0 is the 32-bit word at
// W[n0 + g][k0 + 2t] and b1 the one at W[n0 + g][k0 + 2t + 8].
#pragma once

#include <cuda_bf16.h>

namespace b2g {

constexpr int kMlpIn = 14;     // contact-point features
constexpr int kMlpInPad = 16;  // padded to one k-step
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2;     // normal and tangent impulse (scaled)
constexpr int kMlpOutPad = 8;  // one n-tile

// Device view of the network. W* are bf16 (row major [out][in], padding rows/columns zero), biases
// f32; mu/sigma normalise the raw features (x - mu) / sigma before they are rounded to bf16.
struct MlpView {
    const __nv_bfloat16* W1;  // [64][16]
    const float* b1;          // [64]
    const __nv_bfloat16* W2;  // [64][64]
    const float* b2;          // [64]
    const __nv_bfloat16* W3;  // [8][64]
    const float* b3;          // [8]
    const float* mu;          // [16]
    const float* sigma;       // [16]
};

__device__ __forceinline__ unsigned PackBf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

__device__ __forceinline__ unsigned Ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void Mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Layer with K = 16 inputs and 64 outputs: acc[nt] = A * W^T + b, then ReLU when relu.
__device__ __forceinline__ void MlpLayerK16(float (&acc)[8][4], const unsigned (&a)[4], const __nv_bfloat16* W,
                                            const float* b, int g, int t)
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = b[8 * nt + 2 * t], b1 = b[8 * nt + 2 * t + 1];
        acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        const __nv_bfloat16* row = W + (8 * nt + g) * kMlpInPad;
        Mma16816(acc[nt], a, Ld32(row + 2 * t), Ld32(row + 2 * t + 8));
    }
}

// A fragments (4 k-chunks of 16) of a 16 x 64 activation held as accumulators, ReLU applied.
__device__ __forceinline__ void MlpReluToA(const float (&acc)[8][4], unsigned (&a)[4][4])
{
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        a[j][0] = PackBf16(fmaxf(acc[2 * j][0], 0.0f), fmaxf(acc[2 * j][1], 0.0f));
        a[j][1] = PackBf16(fmaxf(acc[2 * j][2], 0.0f), fmaxf(acc[2 * j][3], 0.0f));
        a[j][2] = PackBf16(fmaxf(acc[2 * j + 1][0], 0.0f), fmaxf(acc[2 * j + 1][1], 0.0f));
        a[j][3] = PackBf16(fmaxf(acc[2 * j + 1][2], 0.0f), fmaxf(acc[2 * j + 1][3], 0.0f));
    }
}

// Layer with K = 64 inputs (A fragments) and 8 * ntiles outputs.
template <int NT>
__device__ __forceinline__ void MlpLayerK64(float (&acc)[NT][4], const unsigned (&a)[4][4], const __nv_bfloat16* W,
                                            const float* b, int g, int t)
{
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float b0 = b[8 * nt + 2 * t], b1 = b[8 * nt + 2 * t + 1];
        acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
        const __nv_bfloat16* row = W + (8 * nt + g) * kMlpHidden;
#pragma unroll
        for (int j = 0; j < 4; ++j) Mma16816(acc[nt], a[j], Ld32(row + 16 * j + 2 * t), Ld32(row + 16 * j + 2 * t + 8));
    }
}

// Forward pass of a 16-row tile for the whole warp. x is the tile's normalised input in bf16,
// row major [16][16] (in shared memory). On return, lanes with t == 0 hold y[g][0..1] in out[0..1]
// and y[g+8][0..1] in out[2..3].
__device__ __forceinline__ void MlpForwardTile(const MlpView& M, const __nv_bfloat16* x, float (&out)[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    unsigned a0[4];
    a0[0] = Ld32(x + g * kMlpInPad + 2 * t);
    a0[1] = Ld32(x + (g + 8) * kMlpInPad + 2 * t);
    a0[2] = Ld32(x + g * kMlpInPad + 2 * t + 8);
    a0[3] = Ld32(x + (g + 8) * kMlpInPad + 2 * t + 8);
    float h[8][4];
    MlpLayerK16(h, a0, M.W1, M.b1, g, t);
    unsigned a1[4][4];
    MlpReluToA(h, a1);
    MlpLayerK64<8>(h, a1, M.W2, M.b2, g, t);
    MlpReluToA(h, a1);
    float y[1][4];
    MlpLayerK64<1>(y, a1, M.W3, M.b3, g, t);
    out[0] = y[0][0]; out[1] = y[0][1]; out[2] = y[0][2]; out[3] = y[0][3];
}

} // namespace b2g
