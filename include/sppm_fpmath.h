/*
 * sppm_fpmath.h -- deterministic single-precision arithmetic shared by the CUDA kernels and the
 * CPU restatement of the glslppm shader path.
 *
 * GLSL 1.20 leaves the precision of sin, cos, pow and exp implementation-defined, and the shader
 * path is chaotic: a one-ulp difference in a photon direction changes which triangle the next
 * segment hits.  To make the GPU path and the CPU checker produce bit-identical photon paths,
 * every transcendental on the path is pinned to the functions below.  They are built only from
 * IEEE-754 single-precision +, -, *, /, floor and integer bit manipulation, evaluated in a fixed
 * order, so a CPU build (compiled with -ffp-contract=off, no -ffast-math) and a CUDA build (device
 * code uses the __f*_rn intrinsics, which are never contracted into FMAs) round identically.
 *
 * Methods (all from the mathematics, constants derived from high-precision pi, ln 2, factorials):
 *  - sin/cos: Cody-Waite additive range reduction by pi/2 (Cody & Waite, "Software Manual for the
 *    Elementary Functions", 1980) with a three-part split of pi/2 whose first two parts carry 12
 *    significant bits (k*P1 and k*P2 are exact for |k| < 4096), then the Taylor series of sin to
 *    r^9 and of cos to r^10 on |r| <= pi/4 (truncation error < 2e-9).  Full accuracy for
 *    |x| < 6400; larger arguments are reduced with growing absolute error.
 *  - log2: x = m * 2^e with m in [sqrt(1/2), sqrt(2)], ln m = 2 atanh(s), s = (m-1)/(m+1), series
 *    to s^11 (|s| <= 0.1716, truncation error < 1e-10).
 *  - exp2: t = k + f with k = floor(t + 1/2), |f| <= 1/2, e^(f ln 2) by its Taylor series to u^7
 *    (|u| <= 0.347, truncation error < 6e-9), scaled by 2^k through the exponent field.
 *  - exp: Cody-Waite reduction by ln 2 (two-part split, 12-bit high part), then the same series.
 *  - pow(x, y) = exp2(y * log2 x); its error grows with |y log2 x| (the rounded exponent).
 * Measured accuracy against double-precision libm is checked by tests/test_fpmath.py.
 */
#ifndef SPPM_FPMATH_H
#define SPPM_FPMATH_H

#include <stdint.h>
#include <math.h>
#if !defined(__CUDACC__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define SPPM_FP_FN static __host__ __device__ __forceinline__
#else
#define SPPM_FP_FN static inline
#endif

/* ---- IEEE single-precision primitives that are never fused ---------------------------------- */
SPPM_FP_FN float sppm_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
SPPM_FP_FN float sppm_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
SPPM_FP_FN float sppm_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
SPPM_FP_FN float sppm_div(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
SPPM_FP_FN float sppm_sqrt(float a) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(a);
#else
    return sqrtf(a);
#endif
}
SPPM_FP_FN uint32_t sppm_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
SPPM_FP_FN float sppm_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
SPPM_FP_FN int sppm_isnan(float x) { return x != x; }

/* ---- constants (float values of the exact quantities, 9 significant digits) ------------------ */
#define SPPM_FP_TWO_OVER_PI 6.366197467e-01f
#define SPPM_FP_PIO2_1 1.570312500e+00f /* pi/2 to 12 bits */
#define SPPM_FP_PIO2_2 4.837512970e-04f /* next 12 bits    */
#define SPPM_FP_PIO2_3 7.549790126e-08f /* remainder       */
#define SPPM_FP_INV_3F 1.666666716e-01f  /* 1/3!  */
#define SPPM_FP_INV_5F 8.333333768e-03f  /* 1/5!  */
#define SPPM_FP_INV_7F 1.984127011e-04f  /* 1/7!  */
#define SPPM_FP_INV_9F 2.755731884e-06f  /* 1/9!  */
#define SPPM_FP_INV_2F 5.000000000e-01f  /* 1/2!  */
#define SPPM_FP_INV_4F 4.166666791e-02f  /* 1/4!  */
#define SPPM_FP_INV_6F 1.388888923e-03f  /* 1/6!  */
#define SPPM_FP_INV_8F 2.480158764e-05f  /* 1/8!  */
#define SPPM_FP_INV_10F 2.755731998e-07f /* 1/10! */
#define SPPM_FP_INV3 3.333333433e-01f
#define SPPM_FP_INV5 2.000000030e-01f
#define SPPM_FP_INV7 1.428571492e-01f
#define SPPM_FP_INV9 1.111111119e-01f
#define SPPM_FP_INV11 9.090909362e-02f
#define SPPM_FP_LOG2E 1.442695022e+00f
#define SPPM_FP_LN2 6.931471825e-01f
#define SPPM_FP_LN2_HI 6.931152344e-01f /* ln 2 to 12 bits */
#define SPPM_FP_LN2_LO 3.194618330e-05f
#define SPPM_FP_SQRT2 1.414213538e+00f

/* sin (phase 0) or cos (phase 1) of x */
SPPM_FP_FN float sppm_sincos_phase(float x, int phase) {
    if (sppm_isnan(x) || x == INFINITY || x == -INFINITY) return sppm_sub(x, x); /* NaN */
    const float k = floorf(sppm_add(sppm_mul(x, SPPM_FP_TWO_OVER_PI), 0.5f));
    float r = sppm_sub(x, sppm_mul(k, SPPM_FP_PIO2_1));
    r = sppm_sub(r, sppm_mul(k, SPPM_FP_PIO2_2));
    r = sppm_sub(r, sppm_mul(k, SPPM_FP_PIO2_3));
    const float r2 = sppm_mul(r, r);
    /* sin r = r + r*r2*(-1/3! + r2*(1/5! + r2*(-1/7! + r2/9!))) */
    float ps = sppm_sub(SPPM_FP_INV_7F, sppm_mul(r2, SPPM_FP_INV_9F));
    ps = sppm_sub(SPPM_FP_INV_5F, sppm_mul(r2, ps));
    ps = sppm_sub(SPPM_FP_INV_3F, sppm_mul(r2, ps));
    const float s = sppm_sub(r, sppm_mul(sppm_mul(r, r2), ps));
    /* cos r = 1 - r2/2! + r2^2*(1/4! - r2*(1/6! - r2*(1/8! - r2/10!))) */
    float pc = sppm_sub(SPPM_FP_INV_8F, sppm_mul(r2, SPPM_FP_INV_10F));
    pc = sppm_sub(SPPM_FP_INV_6F, sppm_mul(r2, pc));
    pc = sppm_sub(SPPM_FP_INV_4F, sppm_mul(r2, pc));
    const float c = sppm_add(sppm_sub(1.0f, sppm_mul(r2, SPPM_FP_INV_2F)), sppm_mul(sppm_mul(r2, r2), pc));
    /* quadrant from k modulo 4 (k is an integral float; reduce in float to stay defined for any k) */
    const float kq = sppm_sub(k, sppm_mul(4.0f, floorf(sppm_mul(k, 0.25f))));
    const int q = ((int)kq + phase) & 3;
    if (q == 0) return s;
    if (q == 1) return c;
    if (q == 2) return -s;
    return -c;
}
SPPM_FP_FN float sppm_fsin(float x) { return sppm_sincos_phase(x, 0); }
SPPM_FP_FN float sppm_fcos(float x) { return sppm_sincos_phase(x, 1); }

SPPM_FP_FN float sppm_flog2(float x) {
    if (sppm_isnan(x) || x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (x == INFINITY) return INFINITY;
    uint32_t bits = sppm_f2u(x);
    int e = 0;
    if (bits < 0x00800000u) { /* subnormal: scale by 2^24 (exact) */
        x = sppm_mul(x, 16777216.0f);
        bits = sppm_f2u(x);
        e = -24;
    }
    e += (int)(bits >> 23) - 127;
    float m = sppm_u2f((bits & 0x007FFFFFu) | 0x3F800000u); /* [1, 2) */
    if (m > SPPM_FP_SQRT2) {
        m = sppm_mul(m, 0.5f);
        e += 1;
    }
    const float s = sppm_div(sppm_sub(m, 1.0f), sppm_add(m, 1.0f));
    const float s2 = sppm_mul(s, s);
    float p = sppm_add(SPPM_FP_INV9, sppm_mul(s2, SPPM_FP_INV11));
    p = sppm_add(SPPM_FP_INV7, sppm_mul(s2, p));
    p = sppm_add(SPPM_FP_INV5, sppm_mul(s2, p));
    p = sppm_add(SPPM_FP_INV3, sppm_mul(s2, p));
    p = sppm_add(1.0f, sppm_mul(s2, p));
    const float ln_m = sppm_mul(sppm_mul(2.0f, s), p);
    return sppm_add((float)e, sppm_mul(ln_m, SPPM_FP_LOG2E));
}

/* e^r * 2^k for |r| <= ln(2)/2 + tiny and an integral k in [-150, 128] */
SPPM_FP_FN float sppm_exp_scaled(float r, float k) {
    float p = sppm_add(SPPM_FP_INV_6F, sppm_mul(r, SPPM_FP_INV_7F));
    p = sppm_add(SPPM_FP_INV_5F, sppm_mul(r, p));
    p = sppm_add(SPPM_FP_INV_4F, sppm_mul(r, p));
    p = sppm_add(SPPM_FP_INV_3F, sppm_mul(r, p));
    p = sppm_add(SPPM_FP_INV_2F, sppm_mul(r, p));
    p = sppm_add(1.0f, sppm_mul(r, p));
    p = sppm_add(1.0f, sppm_mul(r, p));
    const int ki = (int)k;
    if (ki > 127) return sppm_mul(sppm_mul(p, sppm_u2f((uint32_t)(127 + 127) << 23)), 2.0f);
    if (ki >= -126) return sppm_mul(p, sppm_u2f((uint32_t)(ki + 127) << 23));
    /* result below the normal range: an exact scaling, then one rounding into the subnormals */
    return sppm_mul(sppm_mul(p, sppm_u2f((uint32_t)(ki + 64 + 127) << 23)), sppm_u2f((uint32_t)(127 - 64) << 23));
}

SPPM_FP_FN float sppm_fexp2(float t) {
    if (sppm_isnan(t)) return t;
    if (t >= 128.0f) return INFINITY;
    if (t < -150.0f) return 0.0f;
    const float k = floorf(sppm_add(t, 0.5f));
    const float f = sppm_sub(t, k); /* exact, |f| <= 1/2 */
    return sppm_exp_scaled(sppm_mul(f, SPPM_FP_LN2), k);
}

/* e^x with Cody-Waite reduction by ln 2 (12-bit high part, exact products for |k| < 4096) */
SPPM_FP_FN float sppm_fexp(float x) {
    if (sppm_isnan(x)) return x;
    if (x >= 88.72284f) return INFINITY;
    if (x < -103.972084f) return 0.0f;
    const float k = floorf(sppm_add(sppm_mul(x, SPPM_FP_LOG2E), 0.5f));
    const float r = sppm_sub(sppm_sub(x, sppm_mul(k, SPPM_FP_LN2_HI)), sppm_mul(k, SPPM_FP_LN2_LO));
    return sppm_exp_scaled(r, k);
}

SPPM_FP_FN float sppm_fpow(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (sppm_isnan(x) || sppm_isnan(y) || x < 0.0f) return NAN;
    if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
    if (x == INFINITY) return y > 0.0f ? INFINITY : 0.0f;
    return sppm_fexp2(sppm_mul(y, sppm_flog2(x)));
}

#endif /* SPPM_FPMATH_H */
