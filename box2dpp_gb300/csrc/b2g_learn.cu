// Training and standalone inference of the learned warm start's MLP (b2g_mlp.cuh), and its C-ABI.
//
// A training step samples a batch of logged contact points, runs forward and backward passes on the
// tensor cores (mma.sync m16n8k16, bf16 operands, f32 accumulation), reduces the gradients per CTA
// in shared memory and then over CTAs with f32 atomics, and applies Adam to the f32 master weights,
// from which the bf16 operand copies are regenerated. Loss: mean over the batch of the squared error
// summed over the two outputs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/box2d_gb300.h"
#include "b2g_mlp.cuh"

using namespace b2g;

namespace {

// f32 master parameter layout
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * kMlpInPad;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpOutPad * kMlpHidden;
constexpr int kParams = kOffB3 + kMlpOutPad;

// padding entries (inputs 14, 15 of W1; outputs 2..7 of W3 and b3) stay zero
__host__ __device__ inline bool IsPadParam(int i)
{
    if (i >= kOffW1 && i < kOffB1) return (i - kOffW1) % kMlpInPad >= kMlpIn;
    if (i >= kOffW3 && i < kOffB3) return (i - kOffW3) / kMlpHidden >= kMlpOut;
    if (i >= kOffB3) return i - kOffB3 >= kMlpOut;
    return false;
}

constexpr int kTrainWarps = 4;
constexpr int kTrainThreads = 32 * kTrainWarps;

struct WarpTiles {                 // per-warp staging, bf16 row major
    __nv_bfloat16 x[16 * kMlpInPad];
    __nv_bfloat16 h1[16 * kMlpHidden];
    __nv_bfloat16 h2[16 * kMlpHidden];
    __nv_bfloat16 dh2[16 * kMlpHidden];
    __nv_bfloat16 dh1[16 * kMlpHidden];
    __nv_bfloat16 dyT[16 * 16];
};
struct TrainSmem {
    WarpTiles w[kTrainWarps];
    float g[kParams];              // this CTA's gradient partial sums
};

__device__ inline unsigned long long Mix64(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ inline unsigned short Bits(__nv_bfloat16 v) { return *reinterpret_cast<unsigned short*>(&v); }
// two bf16 of one column and consecutive rows r, r + 1 of a row-major tile with `ld` columns
__device__ inline unsigned PackCol(const __nv_bfloat16* tile, int ld, int r, int col)
{
    return (unsigned)Bits(tile[r * ld + col]) | ((unsigned)Bits(tile[(r + 1) * ld + col]) << 16);
}
__device__ inline void St32(__nv_bfloat16* p, unsigned v) { *reinterpret_cast<unsigned*>(p) = v; }

// Sum of a value over the 8 lanes sharing t (lane bits 2..4).
__device__ inline float SumOverG(float v)
{
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

struct TrainArgs {
    const float* x;        // [n][16] normalised features (columns 14, 15 zero)
    const float* t;        // [n][2] targets
    int n;
    const int* rows;       // batch rows (nullptr: sampled from seed/step)
    int batch;             // multiple of 16
    unsigned long long seed;
    int step;
    MlpView M;
    const __nv_bfloat16* W2T;  // [64][64], W2T[k][n] = W2[n][k]
    float* grad;           // [kParams], accumulated
    float* loss;           // accumulated sum of squared errors over the batch
};

__global__ void __launch_bounds__(kTrainThreads) MlpTrainKernel(TrainArgs A)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smraw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    WarpTiles& T = S.w[warp];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) S.g[i] = 0.0f;
    for (int i = lane; i < 16 * 16; i += 32) T.dyT[i] = __float2bfloat16_rn(0.0f);
    __syncthreads();
    const float invB = 1.0f / (float)A.batch;
    float lossAcc = 0.0f;
    const int tiles = A.batch / 16;
    for (int tile = blockIdx.x * kTrainWarps + warp; tile < tiles; tile += gridDim.x * kTrainWarps) {
        // rows of this tile: lane 2r, 2r + 1 load half of row r each
        const int rr = lane >> 1, half = lane & 1;
        const int b = tile * 16 + rr;
        const int row = A.rows ? A.rows[b]
                               : (int)(Mix64(A.seed ^ ((unsigned long long)A.step << 32) ^ (unsigned long long)b) %
                                       (unsigned long long)A.n);
        for (int c = 0; c < 8; ++c) T.x[rr * kMlpInPad + 8 * half + c] = __float2bfloat16_rn(A.x[(size_t)row * kMlpInPad + 8 * half + c]);
        const int rowG = __shfl_sync(0xffffffffu, row, 2 * g), rowG8 = __shfl_sync(0xffffffffu, row, 2 * (g + 8));
        __syncwarp();
        // ---- forward
        unsigned a0[4];
        a0[0] = Ld32(T.x + g * kMlpInPad + 2 * t);
        a0[1] = Ld32(T.x + (g + 8) * kMlpInPad + 2 * t);
        a0[2] = Ld32(T.x + g * kMlpInPad + 2 * t + 8);
        a0[3] = Ld32(T.x + (g + 8) * kMlpInPad + 2 * t + 8);
        float z[8][4];
        MlpLayerK16(z, a0, A.M.W1, A.M.b1, g, t);
        unsigned ah1[4][4];
        MlpReluToA(z, ah1);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            St32(T.h1 + g * kMlpHidden + 16 * j + 2 * t, ah1[j][0]);
            St32(T.h1 + (g + 8) * kMlpHidden + 16 * j + 2 * t, ah1[j][1]);
            St32(T.h1 + g * kMlpHidden + 16 * j + 2 * t + 8, ah1[j][2]);
            St32(T.h1 + (g + 8) * kMlpHidden + 16 * j + 2 * t + 8, ah1[j][3]);
        }
        MlpLayerK64<8>(z, ah1, A.M.W2, A.M.b2, g, t);
        bool pos2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) pos2[nt][q] = z[nt][q] > 0.0f;
        unsigned ah2[4][4];
        MlpReluToA(z, ah2);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            St32(T.h2 + g * kMlpHidden + 16 * j + 2 * t, ah2[j][0]);
            St32(T.h2 + (g + 8) * kMlpHidden + 16 * j + 2 * t, ah2[j][1]);
            St32(T.h2 + g * kMlpHidden + 16 * j + 2 * t + 8, ah2[j][2]);
            St32(T.h2 + (g + 8) * kMlpHidden + 16 * j + 2 * t + 8, ah2[j][3]);
        }
        float y[1][4];
        MlpLayerK64<1>(y, ah2, A.M.W3, A.M.b3, g, t);
        // ---- loss and dy (lanes t == 0 hold outputs 0, 1 of rows g and g + 8)
        float dy0 = 0.0f, dy1 = 0.0f, dy80 = 0.0f, dy81 = 0.0f;
        if (t == 0) {
            const float e0 = y[0][0] - A.t[2 * (size_t)rowG], e1 = y[0][1] - A.t[2 * (size_t)rowG + 1];
            const float e80 = y[0][2] - A.t[2 * (size_t)rowG8], e81 = y[0][3] - A.t[2 * (size_t)rowG8 + 1];
            lossAcc += e0 * e0 + e1 * e1 + e80 * e80 + e81 * e81;
            dy0 = 2.0f * e0 * invB; dy1 = 2.0f * e1 * invB; dy80 = 2.0f * e80 * invB; dy81 = 2.0f * e81 * invB;
            T.dyT[0 * 16 + g] = __float2bfloat16_rn(dy0);
            T.dyT[1 * 16 + g] = __float2bfloat16_rn(dy1);
            T.dyT[0 * 16 + g + 8] = __float2bfloat16_rn(dy80);
            T.dyT[1 * 16 + g + 8] = __float2bfloat16_rn(dy81);
        }
        dy0 = __shfl_sync(0xffffffffu, dy0, 4 * g);
        dy1 = __shfl_sync(0xffffffffu, dy1, 4 * g);
        dy80 = __shfl_sync(0xffffffffu, dy80, 4 * g);
        dy81 = __shfl_sync(0xffffffffu, dy81, 4 * g);
        // db3
        {
            float s0 = SumOverG(t == 0 ? dy0 + dy80 : 0.0f), s1 = SumOverG(t == 0 ? dy1 + dy81 : 0.0f);
            if (lane == 0) { atomicAdd(&S.g[kOffB3 + 0], s0); atomicAdd(&S.g[kOffB3 + 1], s1); }
        }
        // ---- dh2 = (dy W3) * relu'(z2), f32 on the CUDA cores (K = 2)
        float d2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = 8 * nt + 2 * t;
            const float w00 = __bfloat162float(A.M.W3[c]), w01 = __bfloat162float(A.M.W3[c + 1]);
            const float w10 = __bfloat162float(A.M.W3[kMlpHidden + c]), w11 = __bfloat162float(A.M.W3[kMlpHidden + c + 1]);
            d2[nt][0] = pos2[nt][0] ? dy0 * w00 + dy1 * w10 : 0.0f;
            d2[nt][1] = pos2[nt][1] ? dy0 * w01 + dy1 * w11 : 0.0f;
            d2[nt][2] = pos2[nt][2] ? dy80 * w00 + dy81 * w10 : 0.0f;
            d2[nt][3] = pos2[nt][3] ? dy80 * w01 + dy81 * w11 : 0.0f;
            const float c0 = SumOverG(d2[nt][0] + d2[nt][2]), c1 = SumOverG(d2[nt][1] + d2[nt][3]);
            if (g == 0) { atomicAdd(&S.g[kOffB2 + c], c0); atomicAdd(&S.g[kOffB2 + c + 1], c1); }
        }
        unsigned ad2[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ad2[j][0] = PackBf16(d2[2 * j][0], d2[2 * j][1]);
            ad2[j][1] = PackBf16(d2[2 * j][2], d2[2 * j][3]);
            ad2[j][2] = PackBf16(d2[2 * j + 1][0], d2[2 * j + 1][1]);
            ad2[j][3] = PackBf16(d2[2 * j + 1][2], d2[2 * j + 1][3]);
            St32(T.dh2 + g * kMlpHidden + 16 * j + 2 * t, ad2[j][0]);
            St32(T.dh2 + (g + 8) * kMlpHidden + 16 * j + 2 * t, ad2[j][1]);
            St32(T.dh2 + g * kMlpHidden + 16 * j + 2 * t + 8, ad2[j][2]);
            St32(T.dh2 + (g + 8) * kMlpHidden + 16 * j + 2 * t + 8, ad2[j][3]);
        }
        // ---- dh1 = (dh2 W2) * relu'(z1) on the tensor cores: B[k][n] = W2[k][n] = W2T[n][k]
        float d1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            d1[nt][0] = d1[nt][1] = d1[nt][2] = d1[nt][3] = 0.0f;
            const __nv_bfloat16* rowT = A.W2T + (8 * nt + g) * kMlpHidden;
#pragma unroll
            for (int j = 0; j < 4; ++j) Mma16816(d1[nt], ad2[j], Ld32(rowT + 16 * j + 2 * t), Ld32(rowT + 16 * j + 2 * t + 8));
        }
        __syncwarp();
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = 8 * nt + 2 * t;
            // relu'(z1) from the stored activations (a positive f32 stays positive in bf16)
            if (!(__bfloat162float(T.h1[g * kMlpHidden + c]) > 0.0f)) d1[nt][0] = 0.0f;
            if (!(__bfloat162float(T.h1[g * kMlpHidden + c + 1]) > 0.0f)) d1[nt][1] = 0.0f;
            if (!(__bfloat162float(T.h1[(g + 8) * kMlpHidden + c]) > 0.0f)) d1[nt][2] = 0.0f;
            if (!(__bfloat162float(T.h1[(g + 8) * kMlpHidden + c + 1]) > 0.0f)) d1[nt][3] = 0.0f;
            const float c0 = SumOverG(d1[nt][0] + d1[nt][2]), c1 = SumOverG(d1[nt][1] + d1[nt][3]);
            if (g == 0) { atomicAdd(&S.g[kOffB1 + c], c0); atomicAdd(&S.g[kOffB1 + c + 1], c1); }
            St32(T.dh1 + g * kMlpHidden + c, PackBf16(d1[nt][0], d1[nt][1]));
            St32(T.dh1 + (g + 8) * kMlpHidden + c, PackBf16(d1[nt][2], d1[nt][3]));
        }
        __syncwarp();
        // ---- weight gradients on the tensor cores, K = the 16 rows of the tile
        // dW3[o][k] = sum_r dy[r][o] h2[r][k]: A = dyT (rows o), B[r][k] = h2[r][k]
        {
            unsigned a[4];
            a[0] = Ld32(T.dyT + g * 16 + 2 * t);
            a[1] = Ld32(T.dyT + (g + 8) * 16 + 2 * t);
            a[2] = Ld32(T.dyT + g * 16 + 2 * t + 8);
            a[3] = Ld32(T.dyT + (g + 8) * 16 + 2 * t + 8);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                Mma16816(acc, a, PackCol(T.h2, kMlpHidden, 2 * t, 8 * nt + g), PackCol(T.h2, kMlpHidden, 2 * t + 8, 8 * nt + g));
                if (g < kMlpOut) {
                    atomicAdd(&S.g[kOffW3 + g * kMlpHidden + 8 * nt + 2 * t], acc[0]);
                    atomicAdd(&S.g[kOffW3 + g * kMlpHidden + 8 * nt + 2 * t + 1], acc[1]);
                }
            }
        }
        // dW2[n][k] = sum_r dh2[r][n] h1[r][k] and dW1[n][k] = sum_r dh1[r][n] x[r][k]
#pragma unroll 1
        for (int mt = 0; mt < 4; ++mt) {
            unsigned a2[4], a1[4];
            a2[0] = PackCol(T.dh2, kMlpHidden, 2 * t, 16 * mt + g);
            a2[1] = PackCol(T.dh2, kMlpHidden, 2 * t, 16 * mt + g + 8);
            a2[2] = PackCol(T.dh2, kMlpHidden, 2 * t + 8, 16 * mt + g);
            a2[3] = PackCol(T.dh2, kMlpHidden, 2 * t + 8, 16 * mt + g + 8);
            a1[0] = PackCol(T.dh1, kMlpHidden, 2 * t, 16 * mt + g);
            a1[1] = PackCol(T.dh1, kMlpHidden, 2 * t, 16 * mt + g + 8);
            a1[2] = PackCol(T.dh1, kMlpHidden, 2 * t + 8, 16 * mt + g);
            a1[3] = PackCol(T.dh1, kMlpHidden, 2 * t + 8, 16 * mt + g + 8);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                Mma16816(acc, a2, PackCol(T.h1, kMlpHidden, 2 * t, 8 * nt + g), PackCol(T.h1, kMlpHidden, 2 * t + 8, 8 * nt + g));
                float* d = &S.g[kOffW2 + (16 * mt + g) * kMlpHidden + 8 * nt + 2 * t];
                atomicAdd(d, acc[0]);
                atomicAdd(d + 1, acc[1]);
                atomicAdd(d + 8 * kMlpHidden, acc[2]);
                atomicAdd(d + 8 * kMlpHidden + 1, acc[3]);
            }
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                Mma16816(acc, a1, PackCol(T.x, kMlpInPad, 2 * t, 8 * nt + g), PackCol(T.x, kMlpInPad, 2 * t + 8, 8 * nt + g));
                float* d = &S.g[kOffW1 + (16 * mt + g) * kMlpInPad + 8 * nt + 2 * t];
                atomicAdd(d, acc[0]);
                atomicAdd(d + 1, acc[1]);
                atomicAdd(d + 8 * kMlpInPad, acc[2]);
                atomicAdd(d + 8 * kMlpInPad + 1, acc[3]);
            }
        }
        __syncwarp();
    }
    lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, 1);
    lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, 2);
    lossAcc = SumOverG(lossAcc);
    if (lane == 0) atomicAdd(A.loss, lossAcc);
    __syncthreads();
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
        if (!IsPadParam(i) && S.g[i] != 0.0f) atomicAdd(&A.grad[i], S.g[i]);
}

// Adam on the f32 master parameters, then the bf16 operand copies (W1, W2, W2^T, W3).
__global__ void MlpAdamKernel(float* p, const float* grad, float* m, float* v, float lr, float b1c, float b2c,
                              __nv_bfloat16* W1b, __nv_bfloat16* W2b, __nv_bfloat16* W2Tb, __nv_bfloat16* W3b, int apply)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float w = p[i];
    if (apply && !IsPadParam(i)) {
        const float gr = grad[i];
        const float mi = 0.9f * m[i] + 0.1f * gr;
        const float vi = 0.999f * v[i] + 0.001f * gr * gr;
        m[i] = mi;
        v[i] = vi;
        w -= lr * (mi / b1c) / (sqrtf(vi / b2c) + 1e-8f);
        p[i] = w;
    }
    const __nv_bfloat16 wb = __float2bfloat16_rn(w);
    if (i < kOffB1) W1b[i - kOffW1] = wb;
    else if (i >= kOffW2 && i < kOffB2) {
        const int k = i - kOffW2, n = k / kMlpHidden, c = k % kMlpHidden;
        W2b[k] = wb;
        W2Tb[c * kMlpHidden + n] = wb;
    } else if (i >= kOffW3 && i < kOffB3) W3b[i - kOffW3] = wb;
}

// Standalone inference over n rows of normalised features: the in-step tile code.
__global__ void MlpInferKernel(MlpView M, const float* x, int n, float* y)
{
    __shared__ __align__(16) __nv_bfloat16 xs[kTrainWarps][16 * kMlpInPad];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int tiles = (n + 15) / 16;
    for (int tile = blockIdx.x * kTrainWarps + warp; tile < tiles; tile += gridDim.x * kTrainWarps) {
        const int rr = lane >> 1, half = lane & 1, row = tile * 16 + rr;
        for (int c = 0; c < 8; ++c)
            xs[warp][rr * kMlpInPad + 8 * half + c] =
                __float2bfloat16_rn(row < n ? x[(size_t)row * kMlpInPad + 8 * half + c] : 0.0f);
        __syncwarp();
        float out[4];
        MlpForwardTile(M, xs[warp], out);
        if (t == 0) {
            const int r0 = tile * 16 + g, r1 = r0 + 8;
            if (r0 < n) { y[2 * (size_t)r0] = out[0]; y[2 * (size_t)r0 + 1] = out[1]; }
            if (r1 < n) { y[2 * (size_t)r1] = out[2]; y[2 * (size_t)r1 + 1] = out[3]; }
        }
        __syncwarp();
    }
}

} // namespace

struct gb_mlp {
    float* p = nullptr;       // master parameters
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* mu = nullptr;      // [16]
    float* sigma = nullptr;   // [16]
    float* loss = nullptr;    // [1]
    __nv_bfloat16 *W1b = nullptr, *W2b = nullptr, *W2Tb = nullptr, *W3b = nullptr;
    float hmu[kMlpInPad], hsigma[kMlpInPad];
    int adamStep = 0;
};

namespace {

gb_status Cuda(cudaError_t e)
{
    if (e == cudaSuccess) return GB_OK;
    std::fprintf(stderr, "box2d_gb300: CUDA error: %s\n", cudaGetErrorString(e));
    return GB_ERR_CUDA;
}
#define GB_TRY(x)                     \
    do {                              \
        gb_status s_ = Cuda(x);       \
        if (s_ != GB_OK) return s_;   \
    } while (0)

MlpView View(const gb_mlp* m)
{
    MlpView M;
    M.W1 = m->W1b; M.b1 = m->p + kOffB1; M.W2 = m->W2b; M.b2 = m->p + kOffB2; M.W3 = m->W3b; M.b3 = m->p + kOffB3;
    M.mu = m->mu; M.sigma = m->sigma;
    return M;
}

gb_status RefreshCopies(gb_mlp* m)
{
    MlpAdamKernel<<<(kParams + 255) / 256, 256>>>(m->p, m->grad, m->m, m->v, 0.0f, 1.0f, 1.0f, m->W1b, m->W2b, m->W2Tb,
                                                  m->W3b, 0);
    GB_TRY(cudaGetLastError());
    return GB_OK;
}

// (x - mu) / sigma into [n][16] with zero padding columns
std::vector<float> Normalise(const gb_mlp* m, const float* x, int n)
{
    std::vector<float> out((size_t)n * kMlpInPad, 0.0f);
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < kMlpIn; ++c) out[(size_t)r * kMlpInPad + c] = (x[(size_t)r * kMlpIn + c] - m->hmu[c]) / m->hsigma[c];
    return out;
}

template <typename T> struct DevBuf {
    T* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n * sizeof(T)); }
};

gb_status TrainSetup()
{
    static bool done = false;
    if (!done) {
        GB_TRY(cudaFuncSetAttribute(MlpTrainKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem)));
        done = true;
    }
    return GB_OK;
}

gb_status RunGrad(gb_mlp* m, const float* dx, const float* dt, int n, const int* rows, int batch,
                  unsigned long long seed, int step, int ctas)
{
    TrainArgs A;
    A.x = dx; A.t = dt; A.n = n; A.rows = rows; A.batch = batch; A.seed = seed; A.step = step;
    A.M = View(m); A.W2T = m->W2Tb; A.grad = m->grad; A.loss = m->loss;
    GB_TRY(cudaMemsetAsync(m->grad, 0, kParams * sizeof(float)));
    GB_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float)));
    MlpTrainKernel<<<ctas, kTrainThreads, sizeof(TrainSmem)>>>(A);
    GB_TRY(cudaGetLastError());
    return GB_OK;
}

} // namespace

extern "C" {

gb_status gb_mlp_create(unsigned long long seed, gb_mlp** out)
{
    if (!out) return GB_ERR_INVALID;
    *out = nullptr;
    gb_mlp* m = new gb_mlp();
    auto fail = [&](gb_status s) { gb_mlp_destroy(m); return s; };
    if (Cuda(cudaMalloc(&m->p, kParams * sizeof(float))) || Cuda(cudaMalloc(&m->grad, kParams * sizeof(float))) ||
        Cuda(cudaMalloc(&m->m, kParams * sizeof(float))) || Cuda(cudaMalloc(&m->v, kParams * sizeof(float))) ||
        Cuda(cudaMalloc(&m->mu, kMlpInPad * sizeof(float))) || Cuda(cudaMalloc(&m->sigma, kMlpInPad * sizeof(float))) ||
        Cuda(cudaMalloc(&m->loss, sizeof(float))) ||
        Cuda(cudaMalloc(&m->W1b, kMlpHidden * kMlpInPad * sizeof(__nv_bfloat16))) ||
        Cuda(cudaMalloc(&m->W2b, kMlpHidden * kMlpHidden * sizeof(__nv_bfloat16))) ||
        Cuda(cudaMalloc(&m->W2Tb, kMlpHidden * kMlpHidden * sizeof(__nv_bfloat16))) ||
        Cuda(cudaMalloc(&m->W3b, kMlpOutPad * kMlpHidden * sizeof(__nv_bfloat16))))
        return fail(GB_ERR_CUDA);
    // He-uniform initialisation from a seeded SplitMix64 stream; biases zero
    std::vector<float> p(kParams, 0.0f);
    unsigned long long s = seed;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int rows, int cols, int fanIn) {
        const double a = std::sqrt(6.0 / fanIn);
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) {
                const int i = off + r * cols + c;
                const double u = next();
                p[i] = IsPadParam(i) ? 0.0f : (float)((2.0 * u - 1.0) * a);
            }
    };
    fill(kOffW1, kMlpHidden, kMlpInPad, kMlpIn);
    fill(kOffW2, kMlpHidden, kMlpHidden, kMlpHidden);
    fill(kOffW3, kMlpOutPad, kMlpHidden, kMlpHidden);
    for (int c = 0; c < kMlpInPad; ++c) { m->hmu[c] = 0.0f; m->hsigma[c] = 1.0f; }
    if (Cuda(cudaMemcpy(m->p, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice)) ||
        Cuda(cudaMemset(m->m, 0, kParams * sizeof(float))) || Cuda(cudaMemset(m->v, 0, kParams * sizeof(float))) ||
        Cuda(cudaMemcpy(m->mu, m->hmu, sizeof(m->hmu), cudaMemcpyHostToDevice)) ||
        Cuda(cudaMemcpy(m->sigma, m->hsigma, sizeof(m->hsigma), cudaMemcpyHostToDevice)) || RefreshCopies(m) ||
        Cuda(cudaDeviceSynchronize()))
        return fail(GB_ERR_CUDA);
    *out = m;
    return GB_OK;
}

gb_status gb_mlp_destroy(gb_mlp* m)
{
    if (!m) return GB_ERR_INVALID;
    cudaFree(m->p); cudaFree(m->grad); cudaFree(m->m); cudaFree(m->v); cudaFree(m->mu); cudaFree(m->sigma);
    cudaFree(m->loss); cudaFree(m->W1b); cudaFree(m->W2b); cudaFree(m->W2Tb); cudaFree(m->W3b);
    delete m;
    return GB_OK;
}

int gb_mlp_param_count(void) { return kParams; }

gb_status gb_mlp_set_params(gb_mlp* m, const float* params, const float* mu, const float* sigma)
{
    if (!m) return GB_ERR_INVALID;
    if (params) {
        std::vector<float> p(params, params + kParams);
        for (int i = 0; i < kParams; ++i)
            if (IsPadParam(i)) p[i] = 0.0f;
        GB_TRY(cudaMemcpy(m->p, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice));
        GB_TRY(cudaMemset(m->m, 0, kParams * sizeof(float)));
        GB_TRY(cudaMemset(m->v, 0, kParams * sizeof(float)));
        m->adamStep = 0;
    }
    if (mu && sigma) {
        for (int c = 0; c < kMlpInPad; ++c) {
            m->hmu[c] = c < kMlpIn ? mu[c] : 0.0f;
            m->hsigma[c] = c < kMlpIn ? sigma[c] : 1.0f;
            if (!(m->hsigma[c] > 0.0f)) return GB_ERR_INVALID;
        }
        GB_TRY(cudaMemcpy(m->mu, m->hmu, sizeof(m->hmu), cudaMemcpyHostToDevice));
        GB_TRY(cudaMemcpy(m->sigma, m->hsigma, sizeof(m->hsigma), cudaMemcpyHostToDevice));
    }
    gb_status s = RefreshCopies(m);
    if (s != GB_OK) return s;
    GB_TRY(cudaDeviceSynchronize());
    return GB_OK;
}

gb_status gb_mlp_get_params(gb_mlp* m, float* params, float* mu, float* sigma)
{
    if (!m) return GB_ERR_INVALID;
    if (params) GB_TRY(cudaMemcpy(params, m->p, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    if (mu) std::memcpy(mu, m->hmu, kMlpIn * sizeof(float));
    if (sigma) std::memcpy(sigma, m->hsigma, kMlpIn * sizeof(float));
    return GB_OK;
}

gb_status gb_mlp_forward(gb_mlp* m, const float* x, int n, float* y)
{
    if (!m || n < 0 || (n > 0 && (!x || !y))) return GB_ERR_INVALID;
    if (n == 0) return GB_OK;
    std::vector<float> xn = Normalise(m, x, n);
    DevBuf<float> dx, dy;
    GB_TRY(dx.alloc(xn.size()));
    GB_TRY(dy.alloc((size_t)2 * n));
    GB_TRY(cudaMemcpy(dx.p, xn.data(), xn.size() * sizeof(float), cudaMemcpyHostToDevice));
    const int tiles = (n + 15) / 16;
    int ctas = (tiles + kTrainWarps - 1) / kTrainWarps;
    if (ctas > 152 * 8) ctas = 152 * 8;
    MlpInferKernel<<<ctas, kTrainThreads>>>(View(m), dx.p, n, dy.p);
    GB_TRY(cudaGetLastError());
    GB_TRY(cudaMemcpy(y, dy.p, (size_t)2 * n * sizeof(float), cudaMemcpyDeviceToHost));
    return GB_OK;
}

gb_status gb_mlp_gradients(gb_mlp* m, const float* x, const float* t, int n, float* grad, float* loss)
{
    if (!m || n <= 0 || n % 16 != 0 || !x || !t) return GB_ERR_INVALID;
    gb_status s = TrainSetup();
    if (s != GB_OK) return s;
    std::vector<float> xn = Normalise(m, x, n);
    std::vector<int> rows(n);
    for (int i = 0; i < n; ++i) rows[i] = i;
    DevBuf<float> dx, dt;
    DevBuf<int> dr;
    GB_TRY(dx.alloc(xn.size()));
    GB_TRY(dt.alloc((size_t)2 * n));
    GB_TRY(dr.alloc(n));
    GB_TRY(cudaMemcpy(dx.p, xn.data(), xn.size() * sizeof(float), cudaMemcpyHostToDevice));
    GB_TRY(cudaMemcpy(dt.p, t, (size_t)2 * n * sizeof(float), cudaMemcpyHostToDevice));
    GB_TRY(cudaMemcpy(dr.p, rows.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    const int tiles = n / 16;
    int ctas = (tiles + kTrainWarps - 1) / kTrainWarps;
    if (ctas > 152 * 4) ctas = 152 * 4;
    s = RunGrad(m, dx.p, dt.p, n, dr.p, n, 0, 0, ctas);
    if (s != GB_OK) return s;
    if (grad) GB_TRY(cudaMemcpy(grad, m->grad, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    float l = 0.0f;
    GB_TRY(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = l / (float)n;
    return GB_OK;
}

gb_status gb_mlp_train(gb_mlp* m, const float* x, const float* t, int n, int steps, int batch, float lr,
                       unsigned long long seed, float* losses)
{
    if (!m || n <= 0 || !x || !t || steps < 0 || batch <= 0 || batch % 16 != 0 || !(lr > 0.0f)) return GB_ERR_INVALID;
    gb_status s = TrainSetup();
    if (s != GB_OK) return s;
    std::vector<float> xn = Normalise(m, x, n);
    DevBuf<float> dx, dt, dl;
    GB_TRY(dx.alloc(xn.size()));
    GB_TRY(dt.alloc((size_t)2 * n));
    GB_TRY(dl.alloc(steps > 0 ? steps : 1));
    GB_TRY(cudaMemcpy(dx.p, xn.data(), xn.size() * sizeof(float), cudaMemcpyHostToDevice));
    GB_TRY(cudaMemcpy(dt.p, t, (size_t)2 * n * sizeof(float), cudaMemcpyHostToDevice));
    const int tiles = batch / 16;
    int ctas = (tiles + kTrainWarps - 1) / kTrainWarps;
    if (ctas > 152 * 2) ctas = 152 * 2;
    for (int k = 0; k < steps; ++k) {
        s = RunGrad(m, dx.p, dt.p, n, nullptr, batch, seed, k, ctas);
        if (s != GB_OK) return s;
        ++m->adamStep;
        const float b1c = 1.0f - std::pow(0.9f, (float)m->adamStep), b2c = 1.0f - std::pow(0.999f, (float)m->adamStep);
        MlpAdamKernel<<<(kParams + 255) / 256, 256>>>(m->p, m->grad, m->m, m->v, lr, b1c, b2c, m->W1b, m->W2b,
                                                      m->W2Tb, m->W3b, 1);
        GB_TRY(cudaGetLastError());
        GB_TRY(cudaMemcpyAsync(dl.p + k, m->loss, sizeof(float), cudaMemcpyDeviceToDevice));
    }
    GB_TRY(cudaDeviceSynchronize());
    if (losses && steps > 0) {
        GB_TRY(cudaMemcpy(losses, dl.p, steps * sizeof(float), cudaMemcpyDeviceToHost));
        for (int k = 0; k < steps; ++k) losses[k] /= (float)batch;
    }
    return GB_OK;
}

} // extern "C"

// In-step access for the runtime (b2g_api.cu): the device view of a network.
b2g::MlpView b2gMlpView(const gb_mlp* m) { return View(m); }
