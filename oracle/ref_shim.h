/*
 * ref_shim.h - OpenCL C builtins for compiling the reference's rendered
 * McKernel program as C++ on the host CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is prepended to the OpenCL source
 * that the reference's own Python plugins render (xopto/mcml/mc.py:531-626,
 * xopto/mcvox/mc.py) so that the reference kernel arithmetic can run on the
 * CPU as the parity oracle and as the timed CPU baseline.  Nothing in the
 * product links against it.
 *
 * Every builtin maps to the single-precision C library function of the same
 * name (logf, sincosf, powf, ...), so a run of the rendered kernel is the
 * reference algorithm evaluated with IEEE float arithmetic and glibc libm.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cfloat>
#include <cstddef>

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

#define REF_VEC2(T, N) struct N##2 { T x, y; };
#define REF_VEC3(T, N) struct N##3 { T x, y, z, w_; };
#define REF_VEC4(T, N) struct N##4 { T x, y, z, w; };
#define REF_VEC8(T, N) struct N##8 { T s[8]; };
#define REF_VEC16(T, N) struct N##16 { T s[16]; };
#define REF_VECS(T, N) REF_VEC2(T, N) REF_VEC3(T, N) REF_VEC4(T, N) REF_VEC8(T, N) REF_VEC16(T, N)
REF_VECS(float, float)
REF_VECS(double, double)
REF_VECS(int, int)
REF_VECS(unsigned int, uint)
REF_VECS(long, long)
REF_VECS(unsigned long, ulong)
REF_VECS(short, short)
REF_VECS(unsigned short, ushort)
REF_VECS(signed char, char)
REF_VECS(unsigned char, uchar)

#define __kernel extern "C"
#define kernel extern "C"
#define __global
#define __constant
#define __local
#define __private
#define global
#define constant
#define local
#define private_

#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif

/* The work-item id is thread local and set by the caller before each
   McKernel invocation (one invocation per RNG stream). */
static thread_local size_t ref_global_id = 0;
extern "C" void ref_set_global_id(size_t gid) { ref_global_id = gid; }
static inline size_t get_global_id(unsigned) { return ref_global_id; }
static inline size_t get_local_id(unsigned) { return 0; }
static inline size_t get_group_id(unsigned) { return ref_global_id; }
static inline size_t get_local_size(unsigned) { return 1; }
static inline size_t get_global_size(unsigned) { return 1; }

template <class T, class U> static inline T atomic_add(volatile T *p, U v) {
    return __atomic_fetch_add(p, (T)v, __ATOMIC_RELAXED);
}
template <class T> static inline T atomic_inc(volatile T *p) {
    return __atomic_fetch_add(p, (T)1, __ATOMIC_RELAXED);
}
template <class T, class U, class V> static inline T atomic_cmpxchg(volatile T *p, U cmp, V val) {
    T expected = (T)cmp;
    __atomic_compare_exchange_n(p, &expected, (T)val, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
    return expected;
}
template <class T> static inline T atom_inc(volatile T *p) { return atomic_inc(p); }

/* Math builtins: single precision overloads resolve to glibc's *f. */
using std::log; using std::exp; using std::sqrt; using std::sin; using std::cos;
using std::tan; using std::fabs; using std::floor; using std::fmin; using std::fmax;
using std::copysign; using std::asin; using std::acos; using std::atan; using std::atan2;
using std::tanh; using std::cbrt; using std::pow; using std::isinf;
static inline float sincos(float x, float *c) { float s; ::sincosf(x, &s, c); return s; }
static inline double sincos(double x, double *c) { double s; ::sincos(x, &s, c); return s; }
static inline float powr(float x, float y) { return ::powf(x, y); }
static inline float rsqrt(float x) { return 1.0f / ::sqrtf(x); }
static inline float native_log(float x) { return ::logf(x); }
static inline float native_exp(float x) { return ::expf(x); }
static inline float native_sqrt(float x) { return ::sqrtf(x); }
static inline float native_rsqrt(float x) { return 1.0f / ::sqrtf(x); }
static inline float native_divide(float a, float b) { return a / b; }
static inline float native_recip(float x) { return 1.0f / x; }
static inline float native_powr(float x, float y) { return ::powf(x, y); }
static inline float native_sin(float x) { return ::sinf(x); }
static inline float native_cos(float x) { return ::cosf(x); }
static inline float native_tan(float x) { return ::tanf(x); }
static inline float half_log(float x) { return ::logf(x); }
static inline float half_exp(float x) { return ::expf(x); }
static inline float half_sqrt(float x) { return ::sqrtf(x); }
static inline float half_rsqrt(float x) { return 1.0f / ::sqrtf(x); }
static inline float half_divide(float a, float b) { return a / b; }
static inline float half_recip(float x) { return 1.0f / x; }
static inline float half_powr(float x, float y) { return ::powf(x, y); }
static inline float half_sin(float x) { return ::sinf(x); }
static inline float half_cos(float x) { return ::cosf(x); }
static inline float half_tan(float x) { return ::tanf(x); }

/* OpenCL integer and conversion builtins. convert_int/convert_uint use the
   default round-toward-zero mode; out-of-range inputs saturate here. */
static inline int convert_int(float x) {
    if (!(x == x)) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}
static inline unsigned convert_uint(float x) {
    if (!(x == x) || x <= 0.0f) return 0u;
    if (x >= 4294967295.0f) return 4294967295u;
    return (unsigned)x;
}
template <class T> static inline T clamp(T x, T lo, T hi) { return x < lo ? lo : (x > hi ? hi : x); }
static inline float clamp(float x, float lo, float hi) { return ::fminf(::fmaxf(x, lo), hi); }
template <class T> static inline T min(T a, T b) { return b < a ? b : a; }
template <class T> static inline T max(T a, T b) { return a < b ? b : a; }
static inline unsigned mul_hi(unsigned a, unsigned b) { return (unsigned)(((unsigned long)a * b) >> 32); }
static inline unsigned rotate(unsigned x, unsigned b) { b &= 31u; return b ? (x << b) | (x >> (32u - b)) : x; }
