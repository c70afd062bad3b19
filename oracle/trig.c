/*
 * Oracle (test infrastructure only): the project-defined single-precision sine/cosine.
 *
 * The reference rotates bodies with libm's sinf/cosf (b2Rot::Set, Box2DRef/Common/b2Math.h:308-320).
 * glibc's sinf/cosf are not correctly rounded (about 1-3.6% of inputs in [2^-4, 64] differ from the
 * correctly rounded value), and a GPU cannot call glibc. So the project fixes ONE deterministic float
 * sin/cos that the GPU kernels and this oracle evaluate identically, in float arithmetic only (GB300's
 * FP64 is far slower than FP32):
 *
 *   1. k = rint(x * 256/pi); r = x - k*pi/256 as a float-float pair (rh, rl): pi/256 = C1 + C2 + C3,
 *      the products k*C1 and k*C2 made exact with fused multiply-adds, the differences with TwoSum.
 *   2. sin r = r + r^3(-1/6 + r^2/120) and cos r = 1 - r^2/2 + r^4/24 as float-float pairs
 *      (|r| <= pi/512, so the corrections are ~1e-6 relative and float precision suffices for them).
 *   3. sin x = S_j cos r + C_j sin r, cos x = C_j cos r - S_j sin r with the float-float table values
 *      S_j, C_j at j = k mod 512, exact products by fused multiply-add, one final rounding to float.
 *
 * The result is within ~2^-41 of the exact value before the last rounding, so it is the correctly
 * rounded float except for about one input in 10^5. Inputs with |k| >= 2^24 keep the same steps
 * (deterministic, not accurate: such angles are not physical). Compiled with -ffp-contract=off; the
 * only fused operations are the explicit fmaf calls. The GPU copy of these steps lives in the
 * package's CUDA sources; tests check both copies agree bit for bit.
 */
#include <math.h>

#include "trig_table.h"

#define B2O_HIDDEN __attribute__((visibility("hidden")))

static const float kTable[512 * 4] = {B2O_TRIG_TABLE_ROWS};

void b2o_sincosf(float x, float* s_out, float* c_out)
{
    if (x == 0.0f) { *s_out = x; *c_out = 1.0f; return; }
    if (!(fabsf(x) <= 3.40282347e38f)) { *s_out = x - x; *c_out = x - x; return; }
    const float kf = rintf(x * B2O_INV_PIO256);
    const int idx = fabsf(kf) < 16777216.0f ? ((int)kf) & 511 : ((int)fmodf(kf, 512.0f)) & 511;
    /* r = x - k*pi/256 in float-float */
    const float p = kf * B2O_PIO256_1;
    const float pe = fmaf(kf, B2O_PIO256_1, -p);
    const float t = x - p;
    const float q = kf * B2O_PIO256_2;
    const float qe = fmaf(kf, B2O_PIO256_2, -q);
    const float s1 = t - pe;
    const float b1 = s1 - t;
    const float s1e = (t - (s1 - b1)) + (-pe - b1);
    const float s2 = s1 - q;
    const float b2 = s2 - s1;
    const float s2e = (s1 - (s2 - b2)) + (-q - b2);
    const float lo = ((s1e + s2e) - qe) - kf * B2O_PIO256_3;
    const float rh = s2 + lo;
    const float rl = lo - (rh - s2);
    /* sin r, cos r */
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
    /* table */
    const float Sh = kTable[4 * idx], Sl = kTable[4 * idx + 1], Ch = kTable[4 * idx + 2], Cl = kTable[4 * idx + 3];
    /* sin x = S cos r + C sin r */
    const float a1 = Sh * ch;
    const float a1l = fmaf(Sh, ch, -a1) + (Sh * cl + Sl * ch);
    const float a2 = Ch * sh;
    const float a2l = fmaf(Ch, sh, -a2) + (Ch * sl + Cl * sh);
    const float sa = a1 + a2;
    const float b4 = sa - a1;
    const float sae = (a1 - (sa - b4)) + (a2 - b4);
    /* cos x = C cos r - S sin r */
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

float b2o_sinf(float x) { float s, c; b2o_sincosf(x, &s, &c); return s; }
float b2o_cosf(float x) { float s, c; b2o_sincosf(x, &s, &c); return c; }

#ifdef B2O_OVERRIDE_LIBM
/* Linked (hidden) into a build of the reference so that its b2Rot::Set calls resolve to the project
 * trig instead of glibc's, changing nothing else in the reference's object code. */
B2O_HIDDEN float sinf(float x) { return b2o_sinf(x); }
B2O_HIDDEN float cosf(float x) { return b2o_cosf(x); }
B2O_HIDDEN void sincosf(float x, float* s, float* c) { b2o_sincosf(x, s, c); }
#endif
