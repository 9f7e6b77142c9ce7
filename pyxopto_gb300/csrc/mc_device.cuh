/*
 * mc_device.cuh - device functions shared by the layered (mcml) and
 * voxelized (mcvox) transport kernels: random numbers, boundary optics,
 * direction sampling, phase functions and integer tallies.
 *
 * Included by the translation units of each math mode:
 *   transport_exact_*.cu, batched_exact.cu
 *                       MCGB_FAST_MATH == 0, compiled with -fmad=false:
 *                       IEEE +,-,*,/,sqrt and the portable log/exp/sincos/powr
 *                       routines, bit-identical to a CPU evaluation.
 *   transport_fast_*.cu, batched.cu
 *                       MCGB_FAST_MATH == 1, compiled with -use_fast_math:
 *                       special-function-unit log2/sin/cos/ex2, approximate
 *                       division and square root (the reference's
 *                       MC_USE_NATIVE_MATH, xopto/mcbase/kernel/mcbase.template.h:522-556).
 * Each unit wraps the kernels in its own namespace (mcgb_exact / mcgb_fast).
 *
 * The algorithms follow PyXOpto's OpenCL device library; each function cites
 * the reference lines it implements.
 */
#pragma once
#include <cstdint>
#include <cfloat>
#include "../../include/xopto_gb300.h"
#include "portable_math.h"

#ifndef MCGB_FAST_MATH
#error "MCGB_FAST_MATH must be defined to 0 or 1"
#endif

#define MCGB_DEV static __device__ __forceinline__

#if MCGB_FAST_MATH
MCGB_DEV float mc_log(float x) { return __logf(x); }
MCGB_DEV float mc_exp(float x) { return __expf(x); }
MCGB_DEV float mc_pow(float x, float y) { return __powf(x, y); }
MCGB_DEV float mc_cbrt(float x) { return cbrtf(x); }
MCGB_DEV void mc_sincos(float x, float *s, float *c) { __sincosf(x, s, c); }
MCGB_DEV float mc_div(float a, float b) { return __fdividef(a, b); }
MCGB_DEV float mc_sqrt(float x) { return sqrtf(x); }
MCGB_DEV float mc_rcp_length(float x2) { return rsqrtf(x2); }
#else
MCGB_DEV float mc_log(float x) { return pm_logf(x); }
MCGB_DEV float mc_exp(float x) { return pm_expf(x); }
MCGB_DEV float mc_pow(float x, float y) { return pm_powrf(x, y); }
MCGB_DEV float mc_cbrt(float x) { return pm_cbrtf(x); }
MCGB_DEV void mc_sincos(float x, float *s, float *c) { pm_sincosf(x, s, c); }
MCGB_DEV float mc_div(float a, float b) { return a / b; }
MCGB_DEV float mc_sqrt(float x) { return sqrtf(x); }
/* mc_normalize_fpv3: k = 1/length (xopto/mcbase/kernel/mcbase.template.c:975-981) */
MCGB_DEV float mc_rcp_length(float x2) { return 1.0f / sqrtf(x2); }
#endif

struct f3 { float x, y, z; };
struct i3 { int x, y, z; };

/* Float-to-int conversions round toward zero and saturate (the reference's
   convert_int / convert_uint). */
MCGB_DEV int cvt_int(float x) { return __float2int_rz(x); }
MCGB_DEV unsigned cvt_uint(float x) { return __float2uint_rz(x); }
MCGB_DEV int fsign(float x) { return x >= 0.0f ? 1 : -1; }
MCGB_DEV int clip_i(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* Marsaglia multiply-with-carry step and its uniform float:
   fp_random_single, xopto/mcbase/kernel/mcbase.template.c:1576-1594.
   x = lo32(x)*a + hi32(x) is one 32x32->64 multiply-add; the float is
   (uint32)x / 2^32 (an exact scaling). */
struct Rng {
    uint64_t x;
    uint32_t a;
    __device__ __forceinline__ float next() {
        x = (uint64_t)(uint32_t)x * (uint64_t)a + (x >> 32);
        return __uint2float_rn((uint32_t)x) * 2.3283064365386963e-10f;
    }
};

MCGB_DEV float dot3(const f3 &a, const f3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* cos_critical, xopto/mcbase/kernel/mcbase.template.c:1229-1231 */
MCGB_DEV float cos_critical(float n1, float n2) {
    return (n1 > n2) ? mc_sqrt(1.0f - mc_div(n2 * n2, n1 * n1)) : 0.0f;
}

/* reflectance, xopto/mcbase/kernel/mcbase.template.c:1244-1289 */
MCGB_DEV float reflectance(float n1, float n2, float cos1, float cc) {
    float R = 1.0f;
    cos1 = fabsf(cos1);
    if (n1 == n2) return 0.0f;
    if (cos1 > cc) {
        float n1_d_n2 = mc_div(n1, n2);
        float sin1 = mc_sqrt(1.0f - cos1 * cos1);
        if (cos1 >= 1.0f) sin1 = 0.0f;
        float sin2 = fminf(1.0f, n1_d_n2 * sin1);
        float cos2 = mc_sqrt(1.0f - sin2 * sin2);
        float n_cos1 = n1_d_n2 * cos1;
        float n_cos2 = n1_d_n2 * cos2;
        float Rs = mc_div(n_cos1 - cos2, n_cos1 + cos2);
        Rs *= Rs;
        float Rp = mc_div(n_cos2 - cos1, n_cos2 + cos1);
        Rp *= Rp;
        R = 0.5f * (Rp + Rs);
        if (cos1 <= 0.0f || sin2 == 1.0f) return 1.0f;
    }
    return R;
}

/* reflectance_cos2: Fresnel reflectance from the cosine of the angle of
   refraction, xopto/mcbase/kernel/mcbase.template.c:1303-1347 */
MCGB_DEV float reflectance_cos2(float n1, float n2, float cos2) {
    cos2 = fabsf(cos2);
    if (n1 == n2) return 0.0f;
    float sin2 = mc_sqrt(1.0f - cos2 * cos2);
    if (cos2 >= 1.0f) sin2 = 0.0f;
    float sin1 = mc_div(n2, n1) * sin2;
    float R = 1.0f;
    if (sin1 < 1.0f) {
        float cos1 = mc_sqrt(1.0f - sin1 * sin1);
        float n1_d_n2 = mc_div(n1, n2);
        float n_cos1 = n1_d_n2 * cos1;
        float n_cos2 = n1_d_n2 * cos2;
        float Rs = mc_div(n_cos1 - cos2, n_cos1 + cos2);
        Rs *= Rs;
        float Rp = mc_div(n_cos2 - cos1, n_cos2 + cos1);
        Rp *= Rp;
        R = 0.5f * (Rp + Rs);
        if (cos1 <= 0.0f || sin2 == 1.0f) return 1.0f;
    }
    return R;
}

/* reflect, xopto/mcbase/kernel/mcbase.template.c:1361-1369 */
MCGB_DEV f3 reflect3(const f3 &p, const f3 &n) {
    float p_n_2 = 2.0f * dot3(p, n);
    return f3{p.x - n.x * p_n_2, p.y - n.y * p_n_2, p.z - n.z * p_n_2};
}

/* refract, xopto/mcbase/kernel/mcbase.template.c:1424-1440 */
MCGB_DEV f3 refract3(const f3 &p, const f3 &n, float n1, float n2) {
    float cos1 = dot3(p, n);
    float n1_d_n2 = mc_div(n1, n2);
    float sin2_squared = n1_d_n2 * n1_d_n2 * (1.0f - cos1 * cos1);
    float k = (float)fsign(cos1) * (n1_d_n2 * fabsf(cos1) - mc_sqrt(1.0f - sin2_squared));
    return f3{n1_d_n2 * p.x - k * n.x, n1_d_n2 * p.y - k * n.y, n1_d_n2 * p.z - k * n.z};
}

/* refract_safe, xopto/mcbase/kernel/mcbase.template.c:1466-1487 */
MCGB_DEV int refract_safe3(const f3 &p, const f3 &n, float n1, float n2, f3 *r) {
    float cos1 = dot3(p, n);
    float n1_d_n2 = mc_div(n1, n2);
    float sin2_squared = n1_d_n2 * n1_d_n2 * (1.0f - cos1 * cos1);
    if (sin2_squared > 1.0f) return 1;
    float k = (float)fsign(cos1) * (n1_d_n2 * fabsf(cos1) - mc_sqrt(1.0f - sin2_squared));
    r->x = n1_d_n2 * p.x - k * n.x;
    r->y = n1_d_n2 * p.y - k * n.y;
    r->z = n1_d_n2 * p.z - k * n.z;
    return 0;
}

/* Free path length -log(u)/mu_t from a per-medium factor stored in the
   shared-memory tables (step sampling, xopto/mcml/kernel/mcml.template.c:528-536).
   EXACT: the factor is 1/mu_t and the step is -log(u)*factor, the
   reference's expression.  FAST: the factor is -ln(2)/mu_t, folded once per
   block, and the step is log2(u)*factor, since log(u) = ln(2)*log2(u). */
#if MCGB_FAST_MATH
MCGB_DEV float step_factor(float inv_mut) { return -0.693147182f * inv_mut; }
MCGB_DEV float sample_step(float u, float factor) { return __log2f(u) * factor; }
#else
MCGB_DEV float step_factor(float inv_mut) { return inv_mut; }
MCGB_DEV float sample_step(float u, float factor) { return -mc_log(u) * factor; }
#endif

/* scatter_direction + unconditional renormalisation,
   xopto/mcbase/kernel/mcbase.template.c:1522-1555.  FAST mode divides by
   sqrt(1 - uz^2) through one reciprocal square root. */
MCGB_DEV void scatter_direction(f3 &dir, float cos_theta, float fi) {
    float sin_fi, cos_fi;
    float sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
    mc_sincos(fi, &sin_fi, &cos_fi);
    float stcf = sin_theta * cos_fi;
    float stsf = sin_theta * sin_fi;
    float px = dir.x;
    if (fabsf(dir.z) >= 1.0f) {
        dir.x = stcf;
        dir.y = stsf;
        dir.z = copysignf(cos_theta, dir.z * cos_theta);
    } else {
#if MCGB_FAST_MATH
        float t = 1.0f - dir.z * dir.z;
        float rk = rsqrtf(t);
        float k = t * rk;
        dir.x = (stcf * px * dir.z - stsf * dir.y) * rk + px * cos_theta;
        dir.y = (stcf * dir.y * dir.z + stsf * px) * rk + dir.y * cos_theta;
#else
        float k = mc_sqrt(1.0f - dir.z * dir.z);
        dir.x = mc_div(stcf * px * dir.z - stsf * dir.y, k) + px * cos_theta;
        dir.y = mc_div(stcf * dir.y * dir.z + stsf * px, k) + dir.y * cos_theta;
#endif
        dir.z = (-stcf) * k + dir.z * cos_theta;
    }
    float k = mc_rcp_length(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    dir.x = dir.x * k;
    dir.y = dir.y * k;
    dir.z = dir.z * k;
}

/* Phase-function constants of one layer/material, precomputed once per
   kernel with the same float operations the per-step formulas use, so the
   sampled values are bit-identical to evaluating the reference formulas in
   place:
     Hg:  pf0 = (g, 1 - g*g, 1 + g*g, 2*g)
     Gk:  pf0 = (g, a, -inv_a, a1), pf1 = (a2, 1 + g*g, 2*g, (1 - g)/(1 + g))
     Lut: pf0 = (a, b, c, (float)(N - 1)), pf1 = (offset, N - 1) as int bits
   FAST math stores 1/(2g) in place of 2g and multiplies (pf_div2g). */
#if MCGB_FAST_MATH
MCGB_DEV float pf_2g(float g) { return 1.0f / (2.0f * g); }
MCGB_DEV float pf_div2g(float x, float c) { return x * c; }
#else
MCGB_DEV float pf_2g(float g) { return 2.0f * g; }
MCGB_DEV float pf_div2g(float x, float c) { return mc_div(x, c); }
#endif
MCGB_DEV void pf_prepare(int kind, const McgbPf &pf, float4 &pf0, float4 &pf1) {
    if (kind == MCGB_PF_HG) {
        float g = pf.p[0];
        pf0 = make_float4(g, 1.0f - g * g, 1.0f + g * g, pf_2g(g));
        pf1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else if (kind == MCGB_PF_GK) {
        float g = pf.p[0];
        pf0 = make_float4(g, pf.p[1], -pf.p[2], pf.p[3]);
        pf1 = make_float4(pf.p[4], 1.0f + g * g, pf_2g(g), mc_div(1.0f - g, 1.0f + g));
    } else if (kind == MCGB_PF_EXT) {
        pf0 = make_float4(pf.p[0], pf.p[1], pf.p[2], pf.p[3]);
        pf1 = make_float4(pf.p[4], __int_as_float((int)pf.lut_offset), 0.0f,
                          __int_as_float((int)pf.ext_kind));
    } else {
        uint32_t n1 = pf.lut_size - 1u;
        pf0 = make_float4(pf.p[0], pf.p[1], pf.p[2], (float)n1);
        pf1 = make_float4(__int_as_float((int)pf.lut_offset), __int_as_float((int)n1), 0.0f, 0.0f);
    }
}

/* Phase-function sampling.  Returns cos(theta) of the new direction about
   the axis ``dir`` and the azimuth, in the reference's order of draws (the
   azimuth first, except for HgDir).  ``dir`` holds the packet's direction
   on entry; HgDir replaces it with the axis it scatters about, the
   phase function's own direction with probability p (the reference's
   mcsim_pf_sample_dir, whose caller rotates that axis).
   Hg:  xopto/mcbase/mcpf/hg.py:80-95
   Gk:  xopto/mcbase/mcpf/gk.py:102-124
   Lut: xopto/mcbase/mcpf/lut.py:125-155
   Ext: Hg2 xopto/mcbase/mcpf/hg2.py:102-130, MHg mhg.py:87-109,
        Pc pc.py:80-92, MPc mpc.py:88-106, MGk mgk.py:110-140,
        Gk2 gk2.py:119-159, Hga hga.py:82-99, HgDir hgdir.py:100-120 */
template <int PF>
MCGB_DEV float pf_sample(const float4 &pf0, const float4 &pf1, const float *lut, Rng &rng,
                         float *azimuth, f3 &dir) {
    if (PF == MCGB_PF_EXT && __float_as_int(pf1.w) == MCGB_PF_EXT_HGDIR) {
        float g = pf0.w;
        float k = mc_div(1.0f - g * g, 1.0f + g * (2.0f * rng.next() - 1.0f));
        float cos_theta = mc_div(1.0f + g * g - k * k, 2.0f * g);
        if (g == 0.0f) cos_theta = 1.0f - 2.0f * rng.next();
        cos_theta = fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        f3 axis = rng.next() < pf1.x ? f3{pf0.x, pf0.y, pf0.z} : dir;
        if (dot3(dir, axis) < 0.0f) cos_theta = -cos_theta;
        dir = axis;
        *azimuth = 6.28318548f * rng.next();
        return cos_theta;
    }
    *azimuth = 6.28318548f * rng.next();
    if (PF == MCGB_PF_HG) {
        float g = pf0.x;
        float k = mc_div(pf0.y, 1.0f + g * (2.0f * rng.next() - 1.0f));
        float cos_theta = pf_div2g(pf0.z - k * k, pf0.w);
        if (g == 0.0f) cos_theta = 1.0f - 2.0f * rng.next();
        return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
    } else if (PF == MCGB_PF_GK) {
        float cos_theta;
        if (pf0.x == 0.0f) {
            cos_theta = 1.0f - 2.0f * rng.next();
        } else if (pf0.y == 0.0f) {
            cos_theta = pf0.w + mc_pow(pf1.w, 2.0f * rng.next()) * pf1.x;
        } else {
            float tmp = pf0.w * rng.next() + pf1.x;
            tmp = pf1.y - mc_pow(tmp, pf0.z);
            cos_theta = pf_div2g(tmp, pf1.z);
        }
        return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
    } else if (PF == MCGB_PF_EXT) {
        int ext = __float_as_int(pf1.w);
        float cos_theta;
        if (ext == MCGB_PF_EXT_HGA) {
            /* Hg with g = dir^T G dir (tensor3f_project,
               xopto/mcbase/kernel/mcbase.template.h:2227-2230) */
            const float *T = lut + __float_as_int(pf1.y);
            float g = dir.x * (T[0] * dir.x + T[1] * dir.y + T[2] * dir.z) +
                      dir.y * (T[3] * dir.x + T[4] * dir.y + T[5] * dir.z) +
                      dir.z * (T[6] * dir.x + T[7] * dir.y + T[8] * dir.z);
            float k = mc_div(1.0f - g * g, 1.0f + g * (2.0f * rng.next() - 1.0f));
            cos_theta = mc_div(1.0f + g * g - k * k, 2.0f * g);
            if (g == 0.0f) cos_theta = 1.0f - 2.0f * rng.next();
            return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        }
        if (ext == MCGB_PF_EXT_GK2) {
            /* the first term when u >= b, else the second */
            const float *q = lut + __float_as_int(pf1.y);
            if (rng.next() < q[10]) q += 5;
            float g = q[0];
            if (g == 0.0f) {
                cos_theta = 1.0f - 2.0f * rng.next();
            } else if (q[1] == 0.0f) {
                cos_theta = q[3] + mc_pow(mc_div(1.0f - g, 1.0f + g), 2.0f * rng.next()) * q[4];
            } else {
                float tmp = q[3] * rng.next() + q[4];
                tmp = 1.0f + g * g - mc_pow(tmp, -q[2]);
                cos_theta = mc_div(tmp, 2.0f * g);
            }
            return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
        }
        if (ext == MCGB_PF_EXT_HG2) {
            /* component 1 when u >= b, else component 2 */
            float g = rng.next() >= pf0.z ? pf0.x : pf0.y;
            float k = mc_div(1.0f - g * g, 1.0f + g * (2.0f * rng.next() - 1.0f));
            cos_theta = mc_div(1.0f + g * g - k * k, 2.0f * g);
            if (g == 0.0f) cos_theta = 1.0f - 2.0f * rng.next();
            return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        }
        if (ext == MCGB_PF_EXT_MGK) {
            if (rng.next() <= pf0.y) {
                float g = pf0.x;
                if (g == 0.0f) {
                    cos_theta = 1.0f - 2.0f * rng.next();
                } else if (pf0.z == 0.0f) {
                    cos_theta = pf0.w + mc_pow(mc_div(1.0f - g, 1.0f + g), 2.0f * rng.next()) * pf1.x;
                } else {
                    float tmp = pf0.w * rng.next() + pf1.x;
                    tmp = 1.0f + g * g - mc_pow(tmp, -pf0.z);
                    cos_theta = mc_div(tmp, 2.0f * g);
                }
            } else {
                cos_theta = mc_cbrt(2.0f * rng.next() - 1.0f);
            }
            return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
        }
        if (ext == MCGB_PF_EXT_PC) {
            cos_theta = 2.0f * mc_pow(rng.next(), mc_div(1.0f, pf0.x + 1.0f)) - 1.0f;
        } else if (rng.next() <= pf0.y) {
            if (ext == MCGB_PF_EXT_MHG) {
                float g = pf0.x;
                float k = mc_div(1.0f - g * g, 1.0f + g * (2.0f * rng.next() - 1.0f));
                cos_theta = mc_div(1.0f + g * g - k * k, 2.0f * g);
                if (g == 0.0f) cos_theta = 1.0f - 2.0f * rng.next();
            } else {
                cos_theta = 2.0f * mc_pow(rng.next(), mc_div(1.0f, pf0.x + 1.0f)) - 1.0f;
            }
        } else {
            /* the (3/2) cos^2 component: cos = cbrt(2u - 1) */
            cos_theta = mc_cbrt(2.0f * rng.next() - 1.0f);
        }
        return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
    } else {
        int offset = __float_as_int(pf1.x);
        int n1 = __float_as_int(pf1.y);
        float fp_index = (mc_div(pf0.x, rng.next() - pf0.z) - pf0.y + 1.0f) * pf0.w * 0.5f;
        float fp_index_floor = floorf(fp_index);
        float d = fp_index - fp_index_floor;
        /* clamped to the table: parameters that map a uniform number
           outside [0, N-1] would read past the table in the reference */
        int index = clip_i(cvt_int(fp_index_floor), 0, n1);
        int i1 = index + 1 < n1 ? index + 1 : n1;
        return lut[offset + index] * (1.0f - d) + lut[offset + i1] * d;
    }
}

/* weight_to_int(w)*accept (xopto/mcml/kernel/mcml.template.h:606) */
MCGB_DEV uint32_t weight_to_u32(float w, float accept) {
    return (uint32_t)((w * (float)MCGB_ACCU_K + 0.5f) * accept);
}

MCGB_DEV void accu_add(uint64_t *accu, uint64_t index, uint32_t w) {
    atomicAdd((unsigned long long *)(accu + index), (unsigned long long)w);
}

/* (x, y, 0) through a 3x3 transformation (mc_transform_fpv3,
   xopto/mcbase/kernel/mcbase.template.c:683-690; the z term is kept so that
   the float operations match the reference). */
MCGB_DEV float2 transform_xy(const float *T, float x, float y) {
    return make_float2(T[0] * x + T[1] * y + T[2] * 0.0f, T[3] * x + T[4] * y + T[5] * 0.0f);
}

MCGB_DEV int probe_pl_index(const McgbDetector &det, float opl) {
    float pl = opl;
    if (det.pl_log_scale) pl = mc_log(fmaxf(pl, 1e-12f));
    return clip_i(cvt_int((pl - det.pl_min) * det.inv_dpl), 0, (int)det.n_pl - 1);
}

/* Linear look-up tables (mc_fp_lut_t, xopto/mcbase/kernel/mcbase.template.h:
   2494-2535).  Both samplers take the lower table entry at the index rounded
   to the nearest integer but interpolate with the fractional part of the
   index, exactly as the reference's macros do.
   lut_sample_rel: position `where` in [0, 1] over the n entries
   (fp_linear_lut_rel_sample); lut_sample: position (where - first) *
   inv_span over the table, `fallback` outside it (fp_linear_lut_sample). */
MCGB_DEV float lut_interp(const float *t, uint32_t n, float fp_index) {
    uint32_t i1 = cvt_uint(fp_index + 0.5f);
    float w2 = fp_index - floorf(fp_index);
    uint32_t i2 = i1 + 1u < n ? i1 + 1u : n - 1u;
    return t[i1] * (1.0f - w2) + t[i2] * w2;
}

MCGB_DEV float lut_sample_rel(const float *t, uint32_t n, float where, float fallback) {
    float fp_index = where * (float)(n - 1u);
    if (cvt_uint(fp_index + 0.5f) < n) return lut_interp(t, n, fp_index);
    return fallback;
}

MCGB_DEV float lut_sample(const float *t, uint32_t n, float first, float inv_span, float where,
                          float fallback) {
    float fp_index = (where - first) * inv_span * (float)(n - 1u);
    if (fp_index >= 0.0f && fp_index <= (float)(n - 1u)) return lut_interp(t, n, fp_index);
    return fallback;
}

/* weight_to_int(weight*sensitivity) of the look-up-table detectors
   (xopto/mcml/kernel/mcml.template.h:606). */
MCGB_DEV uint32_t lut_weight(float weight, float sensitivity) {
    return cvt_uint(weight * sensitivity * (float)MCGB_ACCU_K + 0.5f);
}

/* Collection look-up-table detectors: TotalLut (xopto/mcml/mcdetector/
   total.py:296-323), TotalLutPl (totalpl.py, TotalLutPl) and FiberLutArray
   (probe/fiberlutarray.py:100-200): weight x sensitivity at the |cosine| of
   the exit direction to the detector (fibre) axis; each fibre's table lives
   inside the detector's float table, whose size (n_y) the C ABI checked. */
MCGB_DEV void lut_detector_deposit(const McgbDetector &det, const f3 &pos, const f3 &dir,
                                   float weight, float opl, uint64_t *accu, const float *lut) {
    uint64_t index = 0;
    float sensitivity = 0.0f;
    if (det.kind == MCGB_DET_FIBER_LUT_ARRAY) {
        const float *t = lut + det.table_offset;
        uint32_t fiber = det.n;
        for (uint32_t i = 0; i < det.n; ++i) {
            const float *f = t + (size_t)i * MCGB_DET_LUT_FIBER_FLOATS;
            float2 lp = transform_xy(f, pos.x - f[9], pos.y - f[10]);
            if (lp.x * lp.x + lp.y * lp.y <= f[11]) {
                fiber = i;
                break;
            }
        }
        if (fiber >= det.n) return;
        const float *f = t + (size_t)fiber * MCGB_DET_LUT_FIBER_FLOATS;
        float pz = f[6] * dir.x + f[7] * dir.y + f[8] * dir.z;
        uint32_t n = __float_as_uint(f[14]), rel = __float_as_uint(f[15]);
        if (n >= 1u && rel <= det.n_y && n <= det.n_y - rel)
            sensitivity = lut_sample(t + rel, n, f[12], f[13], fabsf(pz), 0.0f);
        index = fiber;
    } else {
        f3 ddir{det.direction[0], det.direction[1], det.direction[2]};
        sensitivity = lut_sample(lut + det.table_offset, det.n_y, det.r_min, det.inv_dr,
                                 fabsf(dot3(dir, ddir)), 0.0f);
        if (det.kind == MCGB_DET_TOTAL_LUT_PL) {
            float pl = opl;
            if (det.pl_log_scale) pl = mc_log(fmaxf(pl, 1e-12f));
            index = (uint64_t)clip_i(cvt_int((pl - det.pl_min) * det.inv_dpl), 0, (int)det.n_pl - 1);
        }
    }
    uint32_t w = lut_weight(weight, sensitivity);
    if (w > 0) accu_add(accu, det.offset + index, w);
}

/* Fibre-probe detectors: LinearArray (xopto/mcml/mcdetector/probe/
   lineararray.py:103-162), SixAroundOne (sixaroundone.py:103-184; a later
   ring test overrides an earlier hit, as there), FiberArray
   (fiberarray.py:103-162) and their path-length variants (lineararraypl.py,
   sixaroundonepl.py, fiberarraypl.py: bin pl_index*n + fibre). */
MCGB_DEV void probe_deposit(const McgbDetector &det, const f3 &pos, const f3 &dir, float weight,
                            float opl, uint64_t *accu, const float *lut) {
    if (det.kind >= MCGB_DET_TOTAL_LUT) {
        lut_detector_deposit(det, pos, dir, weight, opl, accu, lut);
        return;
    }
    const int base = det.kind >= MCGB_DET_LINEAR_ARRAY_PL ? det.kind - 3 : det.kind;
    const float *t = lut + det.table_offset;
    const float *T = t;
    uint32_t fiber = det.n;
    float cos_min;
    if (base == MCGB_DET_LINEAR_ARRAY) {
        float fx = t[9], fy = t[10];
        for (uint32_t i = 0; i < det.n; ++i) {
            float2 lp = transform_xy(t, pos.x - fx, pos.y - fy);
            if (lp.x * lp.x + lp.y * lp.y <= t[13]) {
                fiber = i;
                break;
            }
            fx += t[11];
            fy += t[12];
        }
        cos_min = t[14];
    } else if (base == MCGB_DET_SIX_AROUND_ONE) {
        float rx = pos.x - t[9], ry = pos.y - t[10];
        float2 lp = transform_xy(t, rx, ry);
        if (lp.x * lp.x + lp.y * lp.y <= t[11]) fiber = 0;
        lp = transform_xy(t, fabsf(rx) - t[12], ry);
        if (lp.x * lp.x + lp.y * lp.y <= t[11]) fiber = (rx >= 0.0f) ? 1 : 4;
        lp = transform_xy(t, fabsf(rx) - t[12] * 0.5f, fabsf(ry) - t[12] * 0.8660254037844386f);
        if (lp.x * lp.x + lp.y * lp.y <= t[11])
            fiber = (rx >= 0.0f) ? ((ry >= 0.0f) ? 2 : 6) : ((ry >= 0.0f) ? 3 : 5);
        cos_min = t[13];
    } else {
        for (uint32_t i = 0; i < det.n; ++i) {
            const float *f = t + (size_t)i * MCGB_DET_FIBER_FLOATS;
            float2 lp = transform_xy(f, pos.x - f[9], pos.y - f[10]);
            if (lp.x * lp.x + lp.y * lp.y <= f[11]) {
                fiber = i;
                break;
            }
        }
        if (fiber >= det.n) return;
        T = t + (size_t)fiber * MCGB_DET_FIBER_FLOATS;
        cos_min = T[12];
    }
    if (fiber >= det.n) return;
    float pz = T[6] * dir.x + T[7] * dir.y + T[8] * dir.z;
    float accept = (float)(cos_min <= fabsf(pz));
    uint64_t index = fiber;
    if (base != det.kind) index += (uint64_t)probe_pl_index(det, opl) * det.n;
    uint32_t w = weight_to_u32(weight, accept);
    if (w > 0) accu_add(accu, det.offset + index, w);
}

/* Surface detector deposit: Total (xopto/mcml/mcdetector/total.py:86-108),
   Radial (radial.py:117-150), TotalPl (totalpl.py:107-135), RadialPl
   (radialpl.py:138-179), Cartesian (cartesian.py:124-157), CartesianPl
   (cartesianpl.py:146-185) and SymmetricX (symmetric.py:124-156); opl is
   the packet's optical path length. */
template <bool PROBES = false>
MCGB_DEV void detector_deposit(const McgbDetector &det, const f3 &pos, const f3 &dir,
                               float weight, float opl, uint64_t *accu,
                               const float *lut = nullptr) {
    if (det.kind == MCGB_DET_NONE) return;
    if (PROBES && det.kind >= MCGB_DET_LINEAR_ARRAY) {
        probe_deposit(det, pos, dir, weight, opl, accu, lut);
        return;
    }
    f3 ddir{det.direction[0], det.direction[1], det.direction[2]};
    float accept = (float)(det.cos_min <= fabsf(dot3(dir, ddir)));
    uint64_t index = 0;
    if (det.kind == MCGB_DET_RADIAL || det.kind == MCGB_DET_RADIAL_PL) {
        float dx = pos.x - det.position[0];
        float dy = pos.y - det.position[1];
        float r = mc_sqrt(dx * dx + dy * dy);
        if (det.log_scale) r = mc_log(fmaxf(r, 1e-12f));
        int r_index = cvt_int((r - det.r_min) * det.inv_dr);
        index = (uint64_t)clip_i(r_index, 0, (int)det.n - 1);
    }
    if (det.kind == MCGB_DET_CARTESIAN || det.kind == MCGB_DET_CARTESIAN_PL) {
        int ix = clip_i(cvt_int((pos.x - det.r_min) * det.inv_dr), 0, (int)det.n - 1);
        int iy = clip_i(cvt_int((pos.y - det.y_min) * det.inv_dy), 0, (int)det.n_y - 1);
        index = (uint64_t)iy * det.n + (uint64_t)ix;
    } else if (det.kind == MCGB_DET_SYMMETRIC_X) {
        float x = fabsf(pos.x - det.position[0]);
        if (det.log_scale) x = mc_log(fmaxf(x, 1e-12f));
        int ix = clip_i(cvt_int((x - det.r_min) * det.inv_dr), 0, (int)det.n - 1);
        index = (pos.x - det.position[0] >= 0.0f) ? (uint64_t)(ix + (int)det.n)
                                                  : (uint64_t)((int)det.n - ix - 1);
    }
    if (det.kind == MCGB_DET_RADIAL_PL || det.kind == MCGB_DET_TOTAL_PL ||
        det.kind == MCGB_DET_CARTESIAN_PL) {
        float pl = opl;
        if (det.pl_log_scale) pl = mc_log(fmaxf(pl, 1e-12f));
        int pl_index = clip_i(cvt_int((pl - det.pl_min) * det.inv_dpl), 0, (int)det.n_pl - 1);
        uint64_t plane = det.kind == MCGB_DET_RADIAL_PL   ? (uint64_t)det.n
                         : det.kind == MCGB_DET_CARTESIAN_PL ? (uint64_t)det.n * det.n_y
                                                            : 1u;
        index += (uint64_t)pl_index * plane;
    }
    uint32_t w = weight_to_u32(weight, accept);
    if (w > 0) accu_add(accu, det.offset + index, w);
}

/* Fluence deposit (xopto/mcbase/mcfluence/fluence.py:103-143) through a
   one-entry per-thread cache: consecutive deposits into the same voxel are
   summed in a register and flushed with one 64-bit atomic when the voxel
   changes (integer sums, so the tally is unchanged).  Voxel numbers are
   32-bit (the C ABI rejects grids of 2^32 - 1 voxels or more); the cache
   holds a pointer to the grid's first tally. */
struct FluenceCache {
    uint64_t *base;
    uint32_t index;
    uint64_t sum;
    __device__ __forceinline__ void flush() {
        if (sum) atomicAdd((unsigned long long *)(base + index), (unsigned long long)sum);
        sum = 0;
    }
    /* Branch-free: the reduction of the previous voxel's sum is predicated
       on a change of voxel, so lanes of a warp do not diverge around it. */
    __device__ __forceinline__ void add(uint32_t i, uint32_t w) {
        const bool miss = i != index;
        const int fire = (miss && sum != 0ull) ? 1 : 0;
        unsigned long long *addr = (unsigned long long *)(base + index);
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.s32 p, %2, 0;\n\t"
            "@p red.global.add.u64 [%0], %1;\n\t}\n" ::"l"(addr),
            "l"((unsigned long long)sum), "r"(fire)
            : "memory");
        index = miss ? i : index;
        sum = (miss ? 0ull : sum) + w;
    }
};

MCGB_DEV FluenceCache fluence_cache(const McgbFluence &fl, uint64_t *accu) {
    return FluenceCache{accu + fl.offset, 0xFFFFFFFFu, 0ull};
}

/* RATE = false compiles out the fluence-rate scaling: the launcher sends
   rate-mode tallies to the kernels with the optional features (XTRA). */
template <bool RATE = true>
MCGB_DEV void fluence_deposit(const McgbFluence &fl, const f3 &pos, float weight, float mua,
                              FluenceCache &cache) {
#if MCGB_FAST_MATH
    /* one multiply-add per axis; the offsets are loop invariants */
    float ix = fmaf(pos.x, fl.inv_step[0], -fl.top_left[0] * fl.inv_step[0]);
    float iy = fmaf(pos.y, fl.inv_step[1], -fl.top_left[1] * fl.inv_step[1]);
    float iz = fmaf(pos.z, fl.inv_step[2], -fl.top_left[2] * fl.inv_step[2]);
#else
    float ix = (pos.x - fl.top_left[0]) * fl.inv_step[0];
    float iy = (pos.y - fl.top_left[1]) * fl.inv_step[1];
    float iz = (pos.z - fl.top_left[2]) * fl.inv_step[2];
#endif
    /* The reference accepts 0 <= indexf < shape and truncates.  With floor
       conversion (saturating), 0 <= indexf < shape  <=>  0 <= floor(indexf)
       < shape, and floor equals truncation there, so one unsigned compare
       per axis is the same test. */
    uint32_t jx = (uint32_t)__float2int_rd(ix);
    uint32_t jy = (uint32_t)__float2int_rd(iy);
    uint32_t jz = (uint32_t)__float2int_rd(iz);
    if (jx < fl.shape[0] && jy < fl.shape[1] && jz < fl.shape[2]) {
        uint32_t index = (jz * fl.shape[1] + jy) * fl.shape[0] + jx;
        if (RATE && fl.kind == MCGB_FLUENCE_RATE) weight *= (mua != 0.0f) ? mc_div(1.0f, mua) : 0.0f;
        uint32_t w = (uint32_t)(weight * (float)fl.k + 0.5f);
        cache.add(index, w);
    }
}

/* Event bits, xopto/mcbase/kernel/mcbase.template.h:640-660 */
#define MCGB_EV_REFLECTION 1u
#define MCGB_EV_REFRACTION 2u
#define MCGB_EV_BOUNDARY_HIT 4u
#define MCGB_EV_LAUNCH 8u
#define MCGB_EV_ABSORPTION 16u
#define MCGB_EV_SCATTERING 32u
#define MCGB_EV_TERMINATED 64u
#define MCGB_EV_ESCAPED 128u

/* Trace event (xopto/mcbase/mctrace.py:541-583): 8 floats per event, the
   last slot is overwritten when the trace is full. */
MCGB_DEV void trace_event(const McgbTrace &tr, uint64_t photon_index, uint32_t &count,
                          uint32_t events, const f3 &pos, const f3 &dir, float w, float opl,
                          float *fbuf) {
    if (tr.event_mask && !(tr.event_mask & events)) return;
    uint32_t ev = count < tr.max_events - 1 ? count : tr.max_events - 1;
    uint64_t p = (uint64_t)ev * MCGB_TRACE_ENTRY_LEN +
                 photon_index * tr.max_events * MCGB_TRACE_ENTRY_LEN + tr.data_offset;
    float4 *dst = reinterpret_cast<float4 *>(fbuf + p);
    if ((p & 3u) == 0) {
        dst[0] = make_float4(pos.x, pos.y, pos.z, dir.x);
        dst[1] = make_float4(dir.y, dir.z, w, opl);
    } else {
        fbuf[p + 0] = pos.x; fbuf[p + 1] = pos.y; fbuf[p + 2] = pos.z;
        fbuf[p + 3] = dir.x; fbuf[p + 4] = dir.y; fbuf[p + 5] = dir.z;
        fbuf[p + 6] = w; fbuf[p + 7] = opl;
    }
    ++count;
}

/* Device wall clock (ns) for the run deadline. */
MCGB_DEV uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
