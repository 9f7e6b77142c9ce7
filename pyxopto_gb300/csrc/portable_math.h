/*
 * portable_math.h - single-precision log, exp, sin/cos and pow built only
 * from IEEE-754 +, -, *, / and integer bit manipulation.
 *
 * The GB300 transport kernels use these routines in their EXACT math mode.
 * Compiled without floating-point contraction (nvcc -fmad=false, gcc
 * -ffp-contract=off) every operation is a correctly rounded IEEE single
 * precision operation, so a GPU thread and a CPU loop that evaluate the same
 * expression produce identical bits.  That makes a packet's whole trajectory,
 * and therefore every integer tally, reproducible across the GPU kernel and
 * a CPU evaluation of the same algorithm.
 *
 * Methods (all textbook, coefficients are exact Taylor coefficients rounded
 * to float, not fitted constants):
 *   log:  x = m*2^e with m in [sqrt(1/2), sqrt(2)); log(m) = 2*atanh(s),
 *         s = (m-1)/(m+1), atanh series to s^11; e*ln2 added with a
 *         two-part (Cody-Waite) ln2.  Max error ~2 ulp.
 *   exp:  x = k*ln2 + r with |r| <= ln2/2 (Cody-Waite), Taylor series of
 *         e^r to r^8, scaled by 2^k through the exponent field.
 *   sincos: x = k*pi/2 + r with a three-part Cody-Waite pi/2 (exact for
 *         |k| < 256, i.e. |x| < ~400), Taylor series of sin r to r^9 and
 *         cos r to r^10 on |r| <= pi/4, quadrant selection from k mod 4.
 *   powr: exp(y*log(x)) for x >= 0 (OpenCL powr domain).
 */
#ifndef XOPTO_GB300_PORTABLE_MATH_H
#define XOPTO_GB300_PORTABLE_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PM_FN static __host__ __device__ __forceinline__
#else
#include <string.h>
#define PM_FN static inline
#endif

PM_FN uint32_t pm_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}

PM_FN float pm_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}

/* Nearest integer of t for |t| < 2^30 (ties away from zero). */
PM_FN int32_t pm_rint(float t) {
    return (int32_t)(t >= 0.0f ? t + 0.5f : t - 0.5f);
}

PM_FN float pm_logf(float x) {
    const float ln2_hi = 0.693145751953125f;       /* 16 significant bits */
    const float ln2_lo = 1.428606765330187e-06f;
    uint32_t u = pm_f2u(x);
    if (x != x) return x;                          /* NaN */
    if (x < 0.0f) return pm_u2f(0x7fc00000u);      /* NaN */
    if (x == 0.0f) return pm_u2f(0xff800000u);     /* -inf */
    if (u == 0x7f800000u) return x;                /* +inf */
    int32_t e = 0;
    if (u < 0x00800000u) {                         /* subnormal: scale by 2^25 */
        x = x * 33554432.0f;
        u = pm_f2u(x);
        e = -25;
    }
    e += (int32_t)(u >> 23) - 127;
    float m = pm_u2f((u & 0x007fffffu) | 0x3f800000u);   /* [1, 2) */
    if (m > 1.41421354f) { m = m * 0.5f; e += 1; }        /* [0.707, 1.414] */
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float p = 0.181818187f;                        /* 2/11 */
    p = p * z + 0.222222224f;                      /* 2/9  */
    p = p * z + 0.285714298f;                      /* 2/7  */
    p = p * z + 0.400000006f;                      /* 2/5  */
    p = p * z + 0.666666687f;                      /* 2/3  */
    float logm = 2.0f * s + (s * z) * p;
    float fe = (float)e;
    return fe * ln2_hi + (fe * ln2_lo + logm);
}

PM_FN float pm_expf(float x) {
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = 1.428606765330187e-06f;
    const float log2e = 1.44269502f;
    if (x != x) return x;
    if (x > 88.7228394f) return pm_u2f(0x7f800000u);
    if (x < -103.972076f) return 0.0f;
    int32_t k = pm_rint(x * log2e);
    float fk = (float)k;
    float r = (x - fk * ln2_hi) - fk * ln2_lo;
    float p = 2.48015876e-05f;                     /* 1/40320 */
    p = p * r + 1.98412701e-04f;                   /* 1/5040  */
    p = p * r + 1.38888892e-03f;                   /* 1/720   */
    p = p * r + 8.33333377e-03f;                   /* 1/120   */
    p = p * r + 4.16666679e-02f;                   /* 1/24    */
    p = p * r + 0.166666672f;                      /* 1/6     */
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    /* scale by 2^k in two exact steps so that subnormal results and
       k = 128 stay representable */
    int32_t k1 = k / 2;
    int32_t k2 = k - k1;
    float s1 = pm_u2f((uint32_t)(k1 + 127) << 23);
    float s2 = pm_u2f((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

PM_FN void pm_sincosf(float x, float *s, float *c) {
    const float two_over_pi = 0.636619747f;
    const float p1 = 1.5703125f;                   /* pi/2 in three parts */
    const float p2 = 4.83870506e-04f;
    const float p3 = -4.37113883e-08f;
    if (x != x || x - x != 0.0f) {                 /* NaN or inf */
        *s = pm_u2f(0x7fc00000u); *c = *s; return;
    }
    int32_t k = pm_rint(x * two_over_pi);
    float fk = (float)k;
    float r = ((x - fk * p1) - fk * p2) - fk * p3;
    float z = r * r;
    float ps = 2.75573188e-06f;                    /* 1/362880 */
    ps = ps * z - 1.98412701e-04f;                 /* 1/5040   */
    ps = ps * z + 8.33333377e-03f;                 /* 1/120    */
    ps = ps * z - 0.166666672f;                    /* 1/6      */
    float sr = r + (r * z) * ps;
    float pc = -2.75573188e-07f;                   /* 1/3628800 */
    pc = pc * z + 2.48015876e-05f;                 /* 1/40320   */
    pc = pc * z - 1.38888892e-03f;                 /* 1/720     */
    pc = pc * z + 4.16666679e-02f;                 /* 1/24      */
    float cr = (1.0f - 0.5f * z) + (z * z) * pc;
    switch (k & 3) {
        case 0: *s = sr;  *c = cr;  break;
        case 1: *s = cr;  *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

PM_FN float pm_powrf(float x, float y) {
    if (x != x || y != y || x < 0.0f) return pm_u2f(0x7fc00000u);
    if (x == 1.0f) return 1.0f;
    if (x == 0.0f) {
        if (y > 0.0f) return 0.0f;
        if (y < 0.0f) return pm_u2f(0x7f800000u);
        return pm_u2f(0x7fc00000u);
    }
    return pm_expf(y * pm_logf(x));
}

/* cbrt: exp(log(|x|)/3) refined by one Newton step y -= (y^3 - |x|)/(3y^2),
   with the sign of x; 0, inf and NaN are returned unchanged. */
PM_FN float pm_cbrtf(float x) {
    if (x == 0.0f || x != x || x - x != 0.0f) return x;
    float s = x < 0.0f ? -x : x;
    float y = pm_expf(pm_logf(s) * 0.333333343f);
    y = y - (y * y * y - s) / (3.0f * y * y);
    return x < 0.0f ? -y : y;
}

#endif /* XOPTO_GB300_PORTABLE_MATH_H */
