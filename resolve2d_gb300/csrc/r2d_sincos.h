/*
 * r2d_sincos.h -- sine and cosine of a single-precision angle, shared by the
 * CUDA kernels and the CPU oracle so that both see the same rotation values.
 *
 * The reference rotates every vector through nmath.rotate2
 * (src/core/nmath.zig:129-136), which calls Zig's std.math.cos / std.math.sin
 * on an f32 angle.  Those come from the toolchain's libm, so the engine's
 * results depend on one transcendental implementation; the broadphase AABBs,
 * SAT axes, projections and contact points of every rectangle go through it.
 * This header is that implementation for this project, written from the
 * mathematics:
 *
 *   1. Cody & Waite additive range reduction (W. J. Cody, W. Waite,
 *      "Software Manual for the Elementary Functions", 1980):
 *        x = k * (pi/2) + r,   k = nearest integer to x * 2/pi,
 *      with pi/2 split into P1 + P2 + P3 (33, 33 and 53 significant bits).
 *      k*P1 and k*P2 are exact for |k| < 2^20, i.e. |x| < ~1.6e6 rad; past
 *      that the result degrades gracefully (still deterministic).
 *   2. The Maclaurin series of sin (to r^17) and cos (to r^18) on
 *      |r| <= pi/4, evaluated by Horner's rule in double precision.  The
 *      truncation error is below 5e-17, so the float result is the correctly
 *      rounded sin/cos except when the exact value lies within ~1e-16 of a
 *      rounding boundary.  The coefficients are (-1)^j / n! rounded to double.
 *   3. Quadrant selection by k mod 4, then one rounding to float.
 *
 * Only IEEE-754 double +, -, * and floor are used, in a fixed order, and the
 * build disables multiply-add contraction on both sides (-ffp-contract=off
 * for g++, --fmad=false for nvcc), so CPU and GPU return identical bits.
 */
#ifndef R2D_SINCOS_H
#define R2D_SINCOS_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define R2D_SC_FN __host__ __device__ __forceinline__
#else
#define R2D_SC_FN static inline
#endif

/* pi/2 = P1 + P2 + P3 (hex literals so the split is exact by construction). */
#define R2D_SC_INV_PIO2 0x1.45f306dc9c883p-1
#define R2D_SC_P1 0x1.921fb54400000p+0
#define R2D_SC_P2 0x1.0b4611a600000p-34
#define R2D_SC_P3 0x1.3198a2e037073p-69

/* (-1)^j / (2j+1)! and (-1)^j / (2j)! rounded to double. */
#define R2D_SC_S3 (-0x1.5555555555555p-3)
#define R2D_SC_S5 0x1.1111111111111p-7
#define R2D_SC_S7 (-0x1.a01a01a01a01ap-13)
#define R2D_SC_S9 0x1.71de3a556c734p-19
#define R2D_SC_S11 (-0x1.ae64567f544e4p-26)
#define R2D_SC_S13 0x1.6124613a86d09p-33
#define R2D_SC_S15 (-0x1.ae7f3e733b81fp-41)
#define R2D_SC_S17 0x1.952c77030ad4ap-49
#define R2D_SC_C2 (-0x1.0000000000000p-1)
#define R2D_SC_C4 0x1.5555555555555p-5
#define R2D_SC_C6 (-0x1.6c16c16c16c17p-10)
#define R2D_SC_C8 0x1.a01a01a01a01ap-16
#define R2D_SC_C10 (-0x1.27e4fb7789f5cp-22)
#define R2D_SC_C12 0x1.1eed8eff8d898p-29
#define R2D_SC_C14 (-0x1.93974a8c07c9dp-37)
#define R2D_SC_C16 0x1.ae7f3e733b81fp-45
#define R2D_SC_C18 (-0x1.6827863b97d97p-53)

/* sin and cos of a double angle to ~1e-16 (used directly by the FP64 oracle
 * and, through r2d_sincosf, by everything that computes in f32). */
R2D_SC_FN void r2d_sincos_d(double x, double *s_out, double *c_out)
{
    if (!(x == x) || x - x != 0.0) { /* NaN or +-inf */
        double nan_v = x - x;
        *s_out = nan_v;
        *c_out = nan_v;
        return;
    }
    if (x == 0.0) { /* keeps the sign of a zero angle: sin(-0) = -0 */
        *s_out = x;
        *c_out = 1.0;
        return;
    }
    double k = floor(x * R2D_SC_INV_PIO2 + 0.5);
    double r = x - k * R2D_SC_P1;
    r = r - k * R2D_SC_P2;
    r = r - k * R2D_SC_P3;
    double z = r * r;

    double ps = R2D_SC_S17;
    ps = ps * z + R2D_SC_S15;
    ps = ps * z + R2D_SC_S13;
    ps = ps * z + R2D_SC_S11;
    ps = ps * z + R2D_SC_S9;
    ps = ps * z + R2D_SC_S7;
    ps = ps * z + R2D_SC_S5;
    ps = ps * z + R2D_SC_S3;
    double sr = r + (r * z) * ps;

    double pc = R2D_SC_C18;
    pc = pc * z + R2D_SC_C16;
    pc = pc * z + R2D_SC_C14;
    pc = pc * z + R2D_SC_C12;
    pc = pc * z + R2D_SC_C10;
    pc = pc * z + R2D_SC_C8;
    pc = pc * z + R2D_SC_C6;
    pc = pc * z + R2D_SC_C4;
    double cr = (1.0 + z * R2D_SC_C2) + (z * z) * pc;

    int64_t q = ((int64_t)k) & 3;
    if (q == 0) { *s_out = sr;  *c_out = cr; }
    else if (q == 1) { *s_out = cr;  *c_out = -sr; }
    else if (q == 2) { *s_out = -sr; *c_out = -cr; }
    else { *s_out = -cr; *c_out = sr; }
}

/* f32 sin/cos as used by nmath.rotate2: evaluated in double, rounded once. */
R2D_SC_FN void r2d_sincosf(float x, float *s_out, float *c_out)
{
    double s, c;
    r2d_sincos_d((double)x, &s, &c);
    *s_out = (float)s;
    *c_out = (float)c;
}

#endif /* R2D_SINCOS_H */
