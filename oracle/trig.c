/*
 * Oracle (test infrastructure only): the project-defined single-precision sine/cosine.
 *
 * The reference rotates bodies with libm's sinf/cosf (b2Rot::Set, Box2DRef/Common/b2Math.h:308-320).
 * glibc's sinf/cosf are not correctly rounded (about 1-3.6% of inputs in [2^-4, 64] differ from the
 * correctly rounded value), and a GPU cannot call glibc. So the project fixes ONE deterministic
 * float sin/cos that both the GPU kernels and this oracle evaluate identically:
 *
 *   1. Cody-Waite reduction in double: k = rint(x * 2/pi), r = ((x - k*P1) - k*P2) - k*P3, with
 *      pi/2 = P1 + P2 + P3, P1 and P2 holding 26 significant bits each so that k*P1 and k*P2 are
 *      exact for |k| < 2^27.
 *   2. Taylor polynomials of sin and cos on |r| <= pi/4 (terms to r^17 and r^18), Horner form,
 *      plain double multiplies and adds (no fused multiply-add, so every platform rounds alike).
 *   3. Quadrant selection by k mod 4, then one rounding to float.
 *
 * The double evaluation error is about 2^-51 relative, so the float result is the correctly rounded
 * one except with probability ~2^-26 per call. Inputs with |x| >= 2^27 are first reduced with an
 * exact fmod by the double nearest 2*pi (deterministic, not accurate: such angles are not physical).
 *
 * This file must be compiled with -ffp-contract=off. The GPU copy of this algorithm lives in the
 * package's CUDA sources; a GPU test checks the two agree bit for bit.
 */
#include <math.h>

#define B2O_HIDDEN __attribute__((visibility("hidden")))

static const double kTwoOverPi = 0x1.45f306dc9c883p-1;
static const double kP1 = 0x1.921fb50000000p+0;
static const double kP2 = 0x1.110b460000000p-26;
static const double kP3 = 0x1.1a62633145c07p-54;
static const double kTwoPi = 0x1.921fb54442d18p+2;

static const double kS3 = -0x1.5555555555555p-3, kS5 = 0x1.1111111111111p-7, kS7 = -0x1.a01a01a01a01ap-13,
                    kS9 = 0x1.71de3a556c734p-19, kS11 = -0x1.ae64567f544e4p-26, kS13 = 0x1.6124613a86d09p-33,
                    kS15 = -0x1.ae7f3e733b81fp-41, kS17 = 0x1.952c77030ad4ap-49;
static const double kC2 = -0.5, kC4 = 0x1.5555555555555p-5, kC6 = -0x1.6c16c16c16c17p-10,
                    kC8 = 0x1.a01a01a01a01ap-16, kC10 = -0x1.27e4fb7789f5cp-22, kC12 = 0x1.1eed8eff8d898p-29,
                    kC14 = -0x1.93974a8c07c9dp-37, kC16 = 0x1.ae7f3e733b81fp-45, kC18 = -0x1.6827863b97d97p-53;

void b2o_sincosf(float xf, float* s_out, float* c_out)
{
    if (xf == 0.0f) { *s_out = xf; *c_out = 1.0f; return; }
    if (!(fabsf(xf) < INFINITY)) { *s_out = xf - xf; *c_out = xf - xf; return; }
    double x = (double)xf;
    if (fabs(x) >= 134217728.0) x = fmod(x, kTwoPi);
    double k = rint(x * kTwoOverPi);
    double r = x - k * kP1;
    r = r - k * kP2;
    r = r - k * kP3;
    double r2 = r * r;
    double ps = kS17;
    ps = ps * r2 + kS15; ps = ps * r2 + kS13; ps = ps * r2 + kS11; ps = ps * r2 + kS9;
    ps = ps * r2 + kS7;  ps = ps * r2 + kS5;  ps = ps * r2 + kS3;
    double sn = r + (r * r2) * ps;
    double pc = kC18;
    pc = pc * r2 + kC16; pc = pc * r2 + kC14; pc = pc * r2 + kC12; pc = pc * r2 + kC10;
    pc = pc * r2 + kC8;  pc = pc * r2 + kC6;  pc = pc * r2 + kC4;  pc = pc * r2 + kC2;
    double cs = 1.0 + r2 * pc;
    long long q = (long long)k & 3;
    double s, c;
    switch (q) {
        case 0: s = sn;  c = cs;  break;
        case 1: s = cs;  c = -sn; break;
        case 2: s = -sn; c = -cs; break;
        default: s = -cs; c = sn; break;
    }
    *s_out = (float)s;
    *c_out = (float)c;
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
