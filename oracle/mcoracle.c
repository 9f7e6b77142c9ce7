/*
 * mcoracle.c - CPU restatement of PyXOpto's Monte Carlo photon-packet
 * transport kernel (McKernel) for layered (mcml) and voxelized (mcvox)
 * media.
 *
 * TEST INFRASTRUCTURE ONLY: this is the parity oracle.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The
 * product (pyxopto_gb300) never links or calls it.
 *
 * Parity pin: compiled with -ffp-contract=off and run in LIBM math mode,
 * this restatement reproduces the reference's own rendered McKernel (built
 * for the CPU by oracle/render_ref.py) bit-for-bit on the same seeds and the
 * same packet-to-stream mapping; tests/golden/ holds tallies produced by that
 * reference build.  In PORTABLE math mode it evaluates log/exp/sincos/powr
 * with pyxopto_gb300/csrc/portable_math.h, the routines of the GPU kernels'
 * EXACT mode, so GPU and CPU tallies can be compared bit-for-bit.
 *
 * Packet-to-stream mapping: stream t simulates packets t, t+T, t+2T, ...
 * (photon_index = that packet number), each to completion.  The reference
 * takes packets from a global atomic counter instead
 * (xopto/mcml/kernel/mcml.template.c:460,790); with one McKernel call per
 * stream and num_packets = that stream's quota the two agree.
 *
 * Every function cites the reference file:line it restates.
 */
#define _GNU_SOURCE 1
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "../include/xopto_gb300.h"
#include "../pyxopto_gb300/csrc/portable_math.h"
#include "../pyxopto_gb300/csrc/batch_rng.h"

#ifdef _OPENMP
#include <omp.h>
#endif

enum { MO_LIBM = 0, MO_PORTABLE = 1 };

typedef struct { float x, y, z; } v3;
typedef struct { int32_t x, y, z; } i3;

/* ---------------------------------------------------------------- math */
/* xopto/mcbase/kernel/mcbase.template.h:558-590 (standard math branch). */
static inline float m_log(int mm, float x) { return mm ? pm_logf(x) : logf(x); }
static inline float m_exp(int mm, float x) { return mm ? pm_expf(x) : expf(x); }
static inline float m_pow(int mm, float x, float y) { return mm ? pm_powrf(x, y) : powf(x, y); }
static inline float m_cbrt(int mm, float x) { return mm ? pm_cbrtf(x) : cbrtf(x); }
static inline void m_sincos(int mm, float x, float *s, float *c) {
    if (mm) pm_sincosf(x, s, c); else sincosf(x, s, c);
}
/* separate mc_sin / mc_cos calls of the reference (UniformBeam) */
static inline void m_sin_cos(int mm, float x, float *s, float *c) {
    if (mm) pm_sincosf(x, s, c); else { *s = sinf(x); *c = cosf(x); }
}

/* convert_int / convert_uint with round-toward-zero and saturation, the
   behaviour of the GPU's float-to-int conversion. */
static inline int32_t cvt_int(float x) {
    if (!(x == x)) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)x;
}
static inline uint32_t cvt_uint(float x) {
    if (!(x == x) || x <= 0.0f) return 0u;
    if (x >= 4294967295.0f) return 4294967295u;
    return (uint32_t)x;
}
static inline int32_t clip_i(int32_t x, int32_t lo, int32_t hi) {
    return x < lo ? lo : (x > hi ? hi : x);
}
/* mc_fsign, xopto/mcbase/kernel/mcbase.template.h:612 */
static inline int32_t fsign(float x) { return x >= 0.0f ? 1 : -1; }

/* ----------------------------------------------------------------- RNG */
/* fp_random_single, xopto/mcbase/kernel/mcbase.template.c:1576-1594
   (MC_USE_ENHANCED_RNG off). */
static inline float rnd(uint64_t *x, uint32_t a) {
    *x = (*x & 0xFFFFFFFFull) * (uint64_t)a + (*x >> 32);
    return (float)(uint32_t)*x / (float)0xFFFFFFFFu;
}

/* ----------------------------------------------------- vector helpers */
/* mc_dot_fpv3 (mcbase.template.c:880-882) */
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* mc_normalize_fpv3 + mc_length_fpv3 (mcbase.template.c:914-916,975-981) */
static inline v3 normalize3(v3 a) {
    float k = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    v3 r = {a.x * k, a.y * k, a.z * k};
    return r;
}

/* --------------------------------------------------- boundary physics */
/* cos_critical, xopto/mcbase/kernel/mcbase.template.c:1229-1231 */
static inline float cos_critical(float n1, float n2) {
    return (n1 > n2) ? sqrtf(1.0f - (n2 * n2) / (n1 * n1)) : 0.0f;
}

/* reflectance, xopto/mcbase/kernel/mcbase.template.c:1244-1289 */
static float reflectance(float n1, float n2, float cos1, float cc) {
    float Rp, Rs, R = 1.0f, n1_d_n2, sin1, sin2, cos2, n_cos1, n_cos2;
    cos1 = fabsf(cos1);
    if (n1 == n2) return 0.0f;
    if (cos1 > cc) {
        n1_d_n2 = n1 / n2;
        sin1 = sqrtf(1.0f - cos1 * cos1);
        if (cos1 >= 1.0f) sin1 = 0.0f;
        sin2 = fminf(1.0f, n1_d_n2 * sin1);
        cos2 = sqrtf(1.0f - sin2 * sin2);
        n_cos1 = n1_d_n2 * cos1;
        n_cos2 = n1_d_n2 * cos2;
        Rs = (n_cos1 - cos2) / (n_cos1 + cos2);
        Rs *= Rs;
        Rp = (n_cos2 - cos1) / (n_cos2 + cos1);
        Rp *= Rp;
        R = 0.5f * (Rp + Rs);
        if (cos1 <= 0.0f || sin2 == 1.0f) return 1.0f;
    }
    return R;
}

/* reflectance_cos2, xopto/mcbase/kernel/mcbase.template.c:1303-1347 */
static float reflectance_cos2(float n1, float n2, float cos2) {
    float Rp, Rs, R = 1.0f, n1_d_n2, sin1, sin2, cos1, n_cos1, n_cos2;
    cos2 = fabsf(cos2);
    if (n1 == n2) return 0.0f;
    sin2 = sqrtf(1.0f - cos2 * cos2);
    if (cos2 >= 1.0f) sin2 = 0.0f;
    sin1 = (n2 / n1) * sin2;
    if (sin1 < 1.0f) {
        cos1 = sqrtf(1.0f - sin1 * sin1);
        n1_d_n2 = n1 / n2;
        n_cos1 = n1_d_n2 * cos1;
        n_cos2 = n1_d_n2 * cos2;
        Rs = (n_cos1 - cos2) / (n_cos1 + cos2);
        Rs *= Rs;
        Rp = (n_cos2 - cos1) / (n_cos2 + cos1);
        Rp *= Rp;
        R = 0.5f * (Rp + Rs);
        if (cos1 <= 0.0f || sin2 == 1.0f) return 1.0f;
    }
    return R;
}

/* reflect, xopto/mcbase/kernel/mcbase.template.c:1361-1369 */
static inline v3 reflect3(v3 p, v3 n) {
    float p_n_2 = 2.0f * dot3(p, n);
    v3 r = {p.x - n.x * p_n_2, p.y - n.y * p_n_2, p.z - n.z * p_n_2};
    return r;
}

/* refract, xopto/mcbase/kernel/mcbase.template.c:1424-1440 */
static inline v3 refract3(v3 p, v3 n, float n1, float n2) {
    float cos1 = dot3(p, n);
    float n1_d_n2 = n1 / n2;
    float sin2_squared = n1_d_n2 * n1_d_n2 * (1.0f - cos1 * cos1);
    float k = (float)fsign(cos1) * (n1_d_n2 * fabsf(cos1) - sqrtf(1.0f - sin2_squared));
    v3 r = {n1_d_n2 * p.x - k * n.x, n1_d_n2 * p.y - k * n.y, n1_d_n2 * p.z - k * n.z};
    return r;
}

/* refract_safe, xopto/mcbase/kernel/mcbase.template.c:1466-1487 */
static inline int refract_safe3(v3 p, v3 n, float n1, float n2, v3 *r) {
    float cos1 = dot3(p, n);
    float n1_d_n2 = n1 / n2;
    float sin2_squared = n1_d_n2 * n1_d_n2 * (1.0f - cos1 * cos1);
    if (sin2_squared > 1.0f) return 1;
    float k = (float)fsign(cos1) * (n1_d_n2 * fabsf(cos1) - sqrtf(1.0f - sin2_squared));
    r->x = n1_d_n2 * p.x - k * n.x;
    r->y = n1_d_n2 * p.y - k * n.y;
    r->z = n1_d_n2 * p.z - k * n.z;
    return 0;
}

/* scatter_direction, xopto/mcbase/kernel/mcbase.template.c:1522-1555 */
static void scatter_direction(int mm, v3 *dir, float cos_theta, float fi) {
    float sin_fi, cos_fi, sin_theta, px, k, stcf, stsf;
    sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
    m_sincos(mm, fi, &sin_fi, &cos_fi);
    stcf = sin_theta * cos_fi;
    stsf = sin_theta * sin_fi;
    px = dir->x;
    if (fabsf(dir->z) >= 1.0f) {
        dir->x = stcf;
        dir->y = stsf;
        dir->z = copysignf(cos_theta, dir->z * cos_theta);
    } else {
        k = sqrtf(1.0f - dir->z * dir->z);
        dir->x = (stcf * px * dir->z - stsf * dir->y) / k + px * cos_theta;
        dir->y = (stcf * dir->y * dir->z + stsf * px) / k + dir->y * cos_theta;
        dir->z = (-stcf) * k + dir->z * cos_theta;
    }
    *dir = normalize3(*dir);
}

/* -------------------------------------------------- phase functions */
/* Returns cos(theta) and the azimuth; draws in the reference's order.
   Hg: xopto/mcbase/mcpf/hg.py:80-95
   Gk: xopto/mcbase/mcpf/gk.py:102-124
   Lut: xopto/mcbase/mcpf/lut.py:125-155
   Hg2: xopto/mcbase/mcpf/hg2.py:102-130    MHg: xopto/mcbase/mcpf/mhg.py:87-109
   Pc:  xopto/mcbase/mcpf/pc.py:80-92       MPc: xopto/mcbase/mcpf/mpc.py:88-106
   MGk: xopto/mcbase/mcpf/mgk.py:110-140
   Gk2: xopto/mcbase/mcpf/gk2.py:119-159   Hga: xopto/mcbase/mcpf/hga.py:82-99
   HgDir: xopto/mcbase/mcpf/hgdir.py:100-120 (mcsim_pf_sample_dir: the
   direction becomes the axis to rotate about, the azimuth is drawn last) */
static float pf_sample(int mm, int kind, const McgbPf *pf, const float *lut,
                       uint64_t *x, uint32_t a, float *azimuth, v3 *dir) {
    float cos_theta;
    if (kind == MCGB_PF_EXT && pf->ext_kind == MCGB_PF_EXT_HGDIR) {
        float g = pf->p[3];
        float k = (1.0f - g * g) / (1.0f + g * (2.0f * rnd(x, a) - 1.0f));
        cos_theta = (1.0f + g * g - k * k) / (2.0f * g);
        if (g == 0.0f) cos_theta = 1.0f - 2.0f * rnd(x, a);
        cos_theta = fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        v3 axis = *dir;
        if (rnd(x, a) < pf->p[4]) {
            axis.x = pf->p[0];
            axis.y = pf->p[1];
            axis.z = pf->p[2];
        }
        if (dot3(*dir, axis) < 0.0f) cos_theta = -cos_theta;
        *dir = axis;
        *azimuth = 6.28318548f * rnd(x, a);
        return cos_theta;
    }
    if (kind == MCGB_PF_HG) {
        float g = pf->p[0];
        *azimuth = 6.28318548f * rnd(x, a);
        float k = (1.0f - g * g) / (1.0f + g * (2.0f * rnd(x, a) - 1.0f));
        cos_theta = (1.0f + g * g - k * k) / (2.0f * g);
        if (g == 0.0f) cos_theta = 1.0f - 2.0f * rnd(x, a);
        return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
    } else if (kind == MCGB_PF_GK) {
        float g = pf->p[0], ga = pf->p[1], inv_a = pf->p[2], a1 = pf->p[3], a2 = pf->p[4];
        float tmp;
        *azimuth = 6.28318548f * rnd(x, a);
        if (g == 0.0f) {
            cos_theta = 1.0f - 2.0f * rnd(x, a);
        } else if (ga == 0.0f) {
            cos_theta = a1 + m_pow(mm, (1.0f - g) / (1.0f + g), 2.0f * rnd(x, a)) * a2;
        } else {
            tmp = a1 * rnd(x, a) + a2;
            tmp = 1.0f + g * g - m_pow(mm, tmp, -inv_a);
            cos_theta = tmp / (2.0f * g);
        }
        /* mc_fclip = clamp = min(max(x, lo), hi) */
        return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
    } else if (kind == MCGB_PF_EXT) {
        *azimuth = 6.28318548f * rnd(x, a);
        if (pf->ext_kind == MCGB_PF_EXT_HGA) {
            /* tensor3f_project, xopto/mcbase/kernel/mcbase.template.h:2227-2230 */
            const float *T = lut + pf->lut_offset;
            v3 p = *dir;
            float g = p.x * (T[0] * p.x + T[1] * p.y + T[2] * p.z) +
                      p.y * (T[3] * p.x + T[4] * p.y + T[5] * p.z) +
                      p.z * (T[6] * p.x + T[7] * p.y + T[8] * p.z);
            float k = (1.0f - g * g) / (1.0f + g * (2.0f * rnd(x, a) - 1.0f));
            cos_theta = (1.0f + g * g - k * k) / (2.0f * g);
            if (g == 0.0f) cos_theta = 1.0f - 2.0f * rnd(x, a);
            return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        }
        if (pf->ext_kind == MCGB_PF_EXT_GK2) {
            const float *q = lut + pf->lut_offset;
            if (rnd(x, a) < q[10]) q += 5;
            float g = q[0];
            if (g == 0.0f) {
                cos_theta = 1.0f - 2.0f * rnd(x, a);
            } else if (q[1] == 0.0f) {
                cos_theta = q[3] + m_pow(mm, (1.0f - g) / (1.0f + g), 2.0f * rnd(x, a)) * q[4];
            } else {
                float tmp = q[3] * rnd(x, a) + q[4];
                tmp = 1.0f + g * g - m_pow(mm, tmp, -q[2]);
                cos_theta = tmp / (2.0f * g);
            }
            return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
        }
        if (pf->ext_kind == MCGB_PF_EXT_HG2) {
            float g = rnd(x, a) >= pf->p[2] ? pf->p[0] : pf->p[1];
            float k = (1.0f - g * g) / (1.0f + g * (2.0f * rnd(x, a) - 1.0f));
            cos_theta = (1.0f + g * g - k * k) / (2.0f * g);
            if (g == 0.0f) cos_theta = 1.0f - 2.0f * rnd(x, a);
            return fmaxf(fminf(cos_theta, 1.0f), -1.0f);
        }
        if (pf->ext_kind == MCGB_PF_EXT_MGK) {
            float g = pf->p[0], inv_a = pf->p[2], a1 = pf->p[3], a2 = pf->p[4];
            if (rnd(x, a) <= pf->p[1]) {
                if (g == 0.0f) {
                    cos_theta = 1.0f - 2.0f * rnd(x, a);
                } else if (inv_a == 0.0f) {
                    cos_theta = a1 + m_pow(mm, (1.0f - g) / (1.0f + g), 2.0f * rnd(x, a)) * a2;
                } else {
                    float tmp = a1 * rnd(x, a) + a2;
                    tmp = 1.0f + g * g - m_pow(mm, tmp, -inv_a);
                    cos_theta = tmp / (2.0f * g);
                }
            } else {
                cos_theta = m_cbrt(mm, 2.0f * rnd(x, a) - 1.0f);
            }
            return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
        }
        if (pf->ext_kind == MCGB_PF_EXT_PC) {
            cos_theta = 2.0f * m_pow(mm, rnd(x, a), 1.0f / (pf->p[0] + 1.0f)) - 1.0f;
        } else if (rnd(x, a) <= pf->p[1]) {
            if (pf->ext_kind == MCGB_PF_EXT_MHG) {
                float g = pf->p[0];
                float k = (1.0f - g * g) / (1.0f + g * (2.0f * rnd(x, a) - 1.0f));
                cos_theta = (1.0f + g * g - k * k) / (2.0f * g);
                if (g == 0.0f) cos_theta = 1.0f - 2.0f * rnd(x, a);
            } else {
                cos_theta = 2.0f * m_pow(mm, rnd(x, a), 1.0f / (pf->p[0] + 1.0f)) - 1.0f;
            }
        } else {
            cos_theta = m_cbrt(mm, 2.0f * rnd(x, a) - 1.0f);
        }
        return fminf(fmaxf(cos_theta, -1.0f), 1.0f);
    } else {
        float la = pf->p[0], lb = pf->p[1], lc = pf->p[2];
        uint32_t offset = pf->lut_offset;
        uint32_t lut_size = pf->lut_size - 1u;
        *azimuth = 6.28318548f * rnd(x, a);
        float fp_index = (la / (rnd(x, a) - lc) - lb + 1.0f) * (float)lut_size * 0.5f;
        float fp_index_floor = floorf(fp_index);
        float d = fp_index - fp_index_floor;
        /* clamped to the table (the GPU kernel does the same; in-range
           indices are unchanged) */
        int32_t index = clip_i(cvt_int(fp_index_floor), 0, (int32_t)lut_size);
        int32_t i1 = index + 1 < (int32_t)lut_size ? index + 1 : (int32_t)lut_size;
        return lut[offset + (uint32_t)index] * (1.0f - d) + lut[offset + (uint32_t)i1] * d;
    }
}

/* ------------------------------------------------------------ tallies */
static inline uint32_t weight_to_u32(float w, float accept) {
    /* weight_to_int(w)*(accept), xopto/mcml/kernel/mcml.template.h:606 */
    return (uint32_t)((w * (float)MCGB_ACCU_K + 0.5f) * accept);
}

/* (x, y, 0) through a 3x3 transformation (mc_transform_fpv3,
   xopto/mcbase/kernel/mcbase.template.c:683-690). */
static inline void xf_xy(const float *T, float x, float y, float *ox, float *oy) {
    *ox = T[0] * x + T[1] * y + T[2] * 0.0f;
    *oy = T[3] * x + T[4] * y + T[5] * 0.0f;
}

/* Linear look-up tables, the reference's fp_linear_lut_rel_sample and
   fp_linear_lut_sample macros (xopto/mcbase/kernel/mcbase.template.h:
   2507-2535): the lower entry is taken at the index rounded to the nearest
   integer, the interpolation weight is the fractional part of the index. */
static float lut_at(const float *t, uint32_t n, float fp_index) {
    uint32_t i1 = cvt_uint(fp_index + 0.5f);
    float w2 = fp_index - floorf(fp_index);
    uint32_t i2 = i1 + 1u < n ? i1 + 1u : n - 1u;
    return t[i1] * (1.0f - w2) + t[i2] * w2;
}

static float lut_rel(const float *t, uint32_t n, float where, float fallback) {
    float fp_index = where * (float)(n - 1u);
    return cvt_uint(fp_index + 0.5f) < n ? lut_at(t, n, fp_index) : fallback;
}

static float lut_abs(const float *t, uint32_t n, float first, float inv_span, float where,
                     float fallback) {
    float fp_index = (where - first) * inv_span * (float)(n - 1u);
    return (fp_index >= 0.0f && fp_index <= (float)(n - 1u)) ? lut_at(t, n, fp_index) : fallback;
}

/* TotalLut (xopto/mcml/mcdetector/total.py:296-323), TotalLutPl (totalpl.py,
   TotalLutPl) and FiberLutArray (probe/fiberlutarray.py:100-200): weight *
   sensitivity, deposited as weight_to_int(weight*sensitivity)
   (xopto/mcml/kernel/mcml.template.h:606). */
static void lut_detector_deposit(int mm, const McgbDetector *det, v3 pos, v3 dir, float weight,
                                 float opl, uint64_t *accu, const float *lut) {
    uint64_t index = 0;
    float sensitivity = 0.0f;
    if (det->kind == MCGB_DET_FIBER_LUT_ARRAY) {
        const float *t = lut + det->table_offset;
        uint32_t fiber = det->n;
        float lx, ly;
        for (uint32_t i = 0; i < det->n; ++i) {
            const float *f = t + (size_t)i * MCGB_DET_LUT_FIBER_FLOATS;
            xf_xy(f, pos.x - f[9], pos.y - f[10], &lx, &ly);
            if (lx * lx + ly * ly <= f[11]) {
                fiber = i;
                break;
            }
        }
        if (fiber >= det->n) return;
        const float *f = t + (size_t)fiber * MCGB_DET_LUT_FIBER_FLOATS;
        float pz = f[6] * dir.x + f[7] * dir.y + f[8] * dir.z;
        uint32_t n, rel;
        memcpy(&n, &f[14], 4);
        memcpy(&rel, &f[15], 4);
        if (n >= 1u && rel <= det->n_y && n <= det->n_y - rel)
            sensitivity = lut_abs(t + rel, n, f[12], f[13], fabsf(pz), 0.0f);
        index = fiber;
    } else {
        float c = fabsf(dir.x * det->direction[0] + dir.y * det->direction[1] +
                        dir.z * det->direction[2]);
        sensitivity = lut_abs(lut + det->table_offset, det->n_y, det->r_min, det->inv_dr, c, 0.0f);
        if (det->kind == MCGB_DET_TOTAL_LUT_PL) {
            float pl = opl;
            if (det->pl_log_scale) pl = m_log(mm, fmaxf(pl, 1e-12f));
            index = (uint64_t)clip_i(cvt_int((pl - det->pl_min) * det->inv_dpl), 0, (int32_t)det->n_pl - 1);
        }
    }
    uint32_t w = cvt_uint(weight * sensitivity * (float)MCGB_ACCU_K + 0.5f);
    if (w > 0) accu[det->offset + index] += w;
}

/* Fibre-probe detectors: LinearArray (xopto/mcml/mcdetector/probe/lineararray.py:103-162),
   SixAroundOne (sixaroundone.py:103-184; a later ring test overrides an earlier hit),
   FiberArray (fiberarray.py:103-162) and the path-length variants (lineararraypl.py,
   sixaroundonepl.py, fiberarraypl.py: bin pl_index*n + fibre). */
static void probe_deposit(int mm, const McgbDetector *det, v3 pos, v3 dir, float weight,
                          float opl, uint64_t *accu, const float *lut) {
    if (det->kind >= MCGB_DET_TOTAL_LUT) {
        lut_detector_deposit(mm, det, pos, dir, weight, opl, accu, lut);
        return;
    }
    int base = det->kind >= MCGB_DET_LINEAR_ARRAY_PL ? det->kind - 3 : det->kind;
    const float *t = lut + det->table_offset;
    const float *T = t;
    uint32_t fiber = det->n;
    float cos_min, lx, ly;
    if (base == MCGB_DET_LINEAR_ARRAY) {
        float fx = t[9], fy = t[10];
        for (uint32_t i = 0; i < det->n; ++i) {
            xf_xy(t, pos.x - fx, pos.y - fy, &lx, &ly);
            if (lx * lx + ly * ly <= t[13]) {
                fiber = i;
                break;
            }
            fx += t[11];
            fy += t[12];
        }
        cos_min = t[14];
    } else if (base == MCGB_DET_SIX_AROUND_ONE) {
        float rx = pos.x - t[9], ry = pos.y - t[10];
        xf_xy(t, rx, ry, &lx, &ly);
        if (lx * lx + ly * ly <= t[11]) fiber = 0;
        xf_xy(t, fabsf(rx) - t[12], ry, &lx, &ly);
        if (lx * lx + ly * ly <= t[11]) fiber = (rx >= 0.0f) ? 1 : 4;
        xf_xy(t, fabsf(rx) - t[12] * 0.5f, fabsf(ry) - t[12] * 0.8660254037844386f, &lx, &ly);
        if (lx * lx + ly * ly <= t[11])
            fiber = (rx >= 0.0f) ? ((ry >= 0.0f) ? 2 : 6) : ((ry >= 0.0f) ? 3 : 5);
        cos_min = t[13];
    } else {
        for (uint32_t i = 0; i < det->n; ++i) {
            const float *f = t + (size_t)i * MCGB_DET_FIBER_FLOATS;
            xf_xy(f, pos.x - f[9], pos.y - f[10], &lx, &ly);
            if (lx * lx + ly * ly <= f[11]) {
                fiber = i;
                break;
            }
        }
        if (fiber >= det->n) return;
        T = t + (size_t)fiber * MCGB_DET_FIBER_FLOATS;
        cos_min = T[12];
    }
    if (fiber >= det->n) return;
    /* transform_point3f_z, xopto/mcbase/kernel/mcbase.template.h:1875-1876 */
    float pz = T[6] * dir.x + T[7] * dir.y + T[8] * dir.z;
    float accept = (float)(cos_min <= fabsf(pz));
    uint64_t index = fiber;
    if (det->kind >= MCGB_DET_LINEAR_ARRAY_PL) {
        float pl = opl;
        if (det->pl_log_scale) pl = m_log(mm, fmaxf(pl, 1e-12f));
        int32_t pl_index = clip_i(cvt_int((pl - det->pl_min) * det->inv_dpl), 0,
                                  (int32_t)det->n_pl - 1);
        index += (uint64_t)pl_index * det->n;
    }
    uint32_t w = weight_to_u32(weight, accept);
    if (w > 0) accu[det->offset + index] += w;
}

/* Surface detector deposit: Total (xopto/mcml/mcdetector/total.py:86-108),
   Radial (radial.py:117-150), TotalPl (totalpl.py:107-135), RadialPl
   (radialpl.py:138-179), Cartesian (cartesian.py:124-157), CartesianPl
   (cartesianpl.py:146-185), SymmetricX (symmetric.py:124-156);
   opl = mcsim_optical_pathlength. */
static void detector_deposit(int mm, const McgbDetector *det, v3 pos, v3 dir,
                             float weight, float opl, uint64_t *accu, const float *lut) {
    if (det->kind == MCGB_DET_NONE) return;
    if (det->kind >= MCGB_DET_LINEAR_ARRAY) {
        probe_deposit(mm, det, pos, dir, weight, opl, accu, lut);
        return;
    }
    v3 ddir = {det->direction[0], det->direction[1], det->direction[2]};
    float accept = (float)(det->cos_min <= fabsf(dot3(dir, ddir)));
    uint64_t index = 0;
    if (det->kind == MCGB_DET_RADIAL || det->kind == MCGB_DET_RADIAL_PL) {
        float dx = pos.x - det->position[0];
        float dy = pos.y - det->position[1];
        float r = sqrtf(dx * dx + dy * dy);
        if (det->log_scale) r = m_log(mm, fmaxf(r, 1e-12f));
        int32_t r_index = cvt_int((r - det->r_min) * det->inv_dr);
        index = (uint64_t)clip_i(r_index, 0, (int32_t)det->n - 1);
    }
    if (det->kind == MCGB_DET_CARTESIAN || det->kind == MCGB_DET_CARTESIAN_PL) {
        int32_t ix = clip_i(cvt_int((pos.x - det->r_min) * det->inv_dr), 0, (int32_t)det->n - 1);
        int32_t iy = clip_i(cvt_int((pos.y - det->y_min) * det->inv_dy), 0, (int32_t)det->n_y - 1);
        index = (uint64_t)iy * det->n + (uint64_t)ix;
    } else if (det->kind == MCGB_DET_SYMMETRIC_X) {
        float xx = fabsf(pos.x - det->position[0]);
        if (det->log_scale) xx = m_log(mm, fmaxf(xx, 1e-12f));
        int32_t ix = clip_i(cvt_int((xx - det->r_min) * det->inv_dr), 0, (int32_t)det->n - 1);
        index = (pos.x - det->position[0] >= 0.0f) ? (uint64_t)(ix + (int32_t)det->n)
                                                   : (uint64_t)((int32_t)det->n - ix - 1);
    }
    if (det->kind == MCGB_DET_RADIAL_PL || det->kind == MCGB_DET_TOTAL_PL ||
        det->kind == MCGB_DET_CARTESIAN_PL) {
        float pl = opl;
        if (det->pl_log_scale) pl = m_log(mm, fmaxf(pl, 1e-12f));
        int32_t pl_index = clip_i(cvt_int((pl - det->pl_min) * det->inv_dpl), 0,
                                  (int32_t)det->n_pl - 1);
        uint64_t plane = det->kind == MCGB_DET_RADIAL_PL   ? (uint64_t)det->n
                         : det->kind == MCGB_DET_CARTESIAN_PL ? (uint64_t)det->n * det->n_y
                                                             : 1u;
        index += (uint64_t)pl_index * plane;
    }
    uint32_t w = weight_to_u32(weight, accept);
    if (w > 0) accu[det->offset + index] += w;
}

/* Fluence deposit, xopto/mcbase/mcfluence/fluence.py:103-143 */
static void fluence_deposit(const McgbFluence *fl, v3 pos, float weight, float mua,
                            uint64_t *accu) {
    float ix = (pos.x - fl->top_left[0]) * fl->inv_step[0];
    float iy = (pos.y - fl->top_left[1]) * fl->inv_step[1];
    float iz = (pos.z - fl->top_left[2]) * fl->inv_step[2];
    if (ix >= 0 && iy >= 0 && iz >= 0 && ix < (float)fl->shape[0] &&
        iy < (float)fl->shape[1] && iz < (float)fl->shape[2]) {
        uint32_t jx = cvt_uint(ix), jy = cvt_uint(iy), jz = cvt_uint(iz);
        uint64_t index = ((uint64_t)jz * fl->shape[1] + jy) * fl->shape[0] + jx;
        if (fl->kind == MCGB_FLUENCE_RATE) weight *= (mua != 0.0f) ? 1.0f / mua : 0.0f;
        uint32_t w = (uint32_t)(weight * (float)fl->k + 0.5f);
        accu[fl->offset + index] += w;
    }
}

/* Trace event, xopto/mcbase/mctrace.py:541-583 */
typedef struct {
    v3 pos, dir;
    float w, opl;
    uint64_t photon_index;
    uint32_t trace_count;
    uint32_t events;
} TraceState;

static void trace_event(const McgbTrace *tr, TraceState *s, float *fbuf) {
    if (tr->event_mask && !(tr->event_mask & s->events)) return;
    uint32_t ev = s->trace_count < tr->max_events - 1 ? s->trace_count : tr->max_events - 1;
    uint64_t pos = (uint64_t)ev * MCGB_TRACE_ENTRY_LEN +
                   s->photon_index * tr->max_events * MCGB_TRACE_ENTRY_LEN + tr->data_offset;
    fbuf[pos++] = s->pos.x; fbuf[pos++] = s->pos.y; fbuf[pos++] = s->pos.z;
    fbuf[pos++] = s->dir.x; fbuf[pos++] = s->dir.y; fbuf[pos++] = s->dir.z;
    fbuf[pos++] = s->w;
    fbuf[pos++] = s->opl;
    s->trace_count++;
}

/* Event bits, xopto/mcbase/kernel/mcbase.template.h:640-660 */
#define EV_REFLECTION 1u
#define EV_REFRACTION 2u
#define EV_BOUNDARY_HIT 4u
#define EV_LAUNCH 8u
#define EV_ABSORPTION 16u
#define EV_SCATTERING 32u
#define EV_TERMINATED 64u
#define EV_ESCAPED 128u

/* ================================================================ mcml */
typedef struct {
    v3 pos, dir;
    float w;
    int32_t layer;
    float opl;
} MlState;

/* mcsim_launch of the fibre sources: UniformFiberNI
   (xopto/mcml/mcsource/fiberni.py:246-290), LambertianFiberNI
   (fiberni.py:485-534), UniformFiber (fiber.py:267-330) and LambertianFiber
   (fiber.py:576-640).  The tilted kinds test pt_mc.z (0 after the move to
   the surface) against the critical cosine before refracting, so their
   direction is never refracted. */
static void mcml_launch_fiber(int mm, const McgbMcmlConfig *c, const float *lut, MlState *s,
                              uint64_t *x, uint32_t a, uint64_t *accu) {
    const McgbSource *src = &c->source;
    int from_lut = src->kind == MCGB_SRC_UNIFORM_FIBER_LUT_NI || src->kind == MCGB_SRC_UNIFORM_FIBER_LUT;
    int tilted = src->kind == MCGB_SRC_UNIFORM_FIBER || src->kind == MCGB_SRC_LAMBERTIAN_FIBER ||
                 src->kind == MCGB_SRC_UNIFORM_FIBER_LUT;
    int lambertian = src->kind == MCGB_SRC_LAMBERTIAN_FIBER_NI ||
                     src->kind == MCGB_SRC_LAMBERTIAN_FIBER;
    float n_sample = c->layers[1].n, n_core = src->clip;
    const float *T = src->transformation;
    float sin_fi, cos_fi, sin_theta, cos_theta, R;
    float r = sqrtf(rnd(x, a)) * src->sigma[0];
    m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
    if (tilted) {
        v3 ps = {r * cos_fi, r * sin_fi, 0.0f}, pm;
        /* mc_transform_fpv3, xopto/mcbase/kernel/mcbase.template.c:380-386 */
        pm.x = T[0] * ps.x + T[1] * ps.y + T[2] * ps.z;
        pm.y = T[3] * ps.x + T[4] * ps.y + T[5] * ps.z;
        pm.z = T[6] * ps.x + T[7] * ps.y + T[8] * ps.z;
        float k = (0.0f - pm.z) / src->direction[2];
        pm.x += k * src->direction[0];
        pm.y += k * src->direction[1];
        s->pos.x = src->position[0] + pm.x;
        s->pos.y = src->position[1] + pm.y;
    } else {
        s->pos.x = src->position[0] + r * cos_fi;
        s->pos.y = src->position[1] + r * sin_fi;
    }
    s->pos.z = 0.0f;
    m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
    if (lambertian) {
        sin_theta = sqrtf(rnd(x, a)) * src->sigma[1];
    } else {
        /* UniformFiberLut(NI): fp_linear_lut_rel_sample of the emission LUT
           (fiber.py:796-797, fiberni.py:625-626) */
        cos_theta = from_lut ? lut_rel(lut + src->lut_offset, src->lut_size, rnd(x, a), 0.0f)
                             : 1.0f - rnd(x, a) * (1.0f - src->sigma[1]);
        sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
    }
    sin_theta = sin_theta / (tilted ? n_core : n_sample);
    cos_theta = sqrtf(1.0f - sin_theta * sin_theta);
    v3 pt = {cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
    if (tilted) {
        v3 d;
        d.x = T[0] * pt.x + T[1] * pt.y + T[2] * pt.z;
        d.y = T[3] * pt.x + T[4] * pt.y + T[5] * pt.z;
        d.z = T[6] * pt.x + T[7] * pt.y + T[8] * pt.z;
        float cc = cos_critical(n_core, n_sample);
        s->dir = d;
        if (from_lut && d.z > cc) {
            /* UniformFiberLut refracts into the sample, fiber.py:806-813 */
            v3 normal = {0.0f, 0.0f, 1.0f};
            s->dir = refract3(d, normal, n_core, n_sample);
        }
        R = reflectance(n_core, n_sample, d.z, cc);
        if (c->specular.kind != MCGB_DET_NONE)
            detector_deposit(mm, &c->specular, s->pos, d, R, 0.0f, accu, NULL);
    } else {
        s->dir = pt;
        R = reflectance_cos2(n_core, n_sample, pt.z);
        if (c->specular.kind != MCGB_DET_NONE) {
            v3 dir_in = {pt.x, pt.y, -pt.z};
            v3 normal = {0.0f, 0.0f, -1.0f};
            v3 d = refract3(dir_in, normal, n_sample, n_core);
            detector_deposit(mm, &c->specular, s->pos, d, R, 0.0f, accu, NULL);
        }
    }
    s->w = 1.0f - R;
}

/* Line.mcsim_launch (xopto/mcml/mcsource/line.py:95-108),
   GaussianBeam.mcsim_launch (xopto/mcml/mcsource/gaussianbeam.py:119-170) and
   the fibre sources (mcml_launch_fiber). */
static void mcml_launch(int mm, const McgbMcmlConfig *c, const float *lut, MlState *s,
                        uint64_t *x, uint32_t a, uint64_t *accu) {
    const McgbSource *src = &c->source;
    if (src->kind == MCGB_SRC_LINE) {
        s->w = 1.0f - src->reflectance;
        s->pos.x = src->position[0]; s->pos.y = src->position[1]; s->pos.z = src->position[2];
        s->dir.x = src->direction[0]; s->dir.y = src->direction[1]; s->dir.z = src->direction[2];
        if (c->specular.kind != MCGB_DET_NONE) {
            v3 d = {src->direction_reflected[0], src->direction_reflected[1],
                    src->direction_reflected[2]};
            detector_deposit(mm, &c->specular, s->pos, d, src->reflectance, 0.0f, accu, NULL);
        }
        s->layer = 1;
    } else if (src->kind == MCGB_SRC_UNIFORM_BEAM) {
        /* UniformBeam.mcsim_launch, xopto/mcml/mcsource/uniformbeam.py:107-146 */
        float rand_sqrt = sqrtf(rnd(x, a));
        float fi = 6.28318548f * rnd(x, a);
        float sin_fi, cos_fi;
        m_sin_cos(mm, fi, &sin_fi, &cos_fi);
        v3 ps = {rand_sqrt * cos_fi * src->sigma[0], rand_sqrt * sin_fi * src->sigma[1], 0.0f}, pm;
        const float *T = src->transformation;
        pm.x = T[0] * ps.x + T[1] * ps.y + T[2] * ps.z;
        pm.y = T[3] * ps.x + T[4] * ps.y + T[5] * ps.z;
        pm.z = T[6] * ps.x + T[7] * ps.y + T[8] * ps.z;
        float k = (0.0f - pm.z) / src->direction[2];
        pm.x += k * src->direction[0];
        pm.y += k * src->direction[1];
        s->pos.x = src->position[0] + pm.x;
        s->pos.y = src->position[1] + pm.y;
        s->pos.z = 0.0f;
        s->dir.x = src->direction[0]; s->dir.y = src->direction[1]; s->dir.z = src->direction[2];
        s->w = 1.0f - src->reflectance;
        s->layer = 1;
        if (c->specular.kind != MCGB_DET_NONE) {
            v3 dir_in = {s->dir.x, s->dir.y, -s->dir.z};
            v3 normal = {0.0f, 0.0f, -1.0f};
            v3 d = refract3(dir_in, normal, c->layers[1].n, c->layers[0].n);
            detector_deposit(mm, &c->specular, s->pos, d, src->reflectance, 0.0f, accu, NULL);
        }
    } else if (src->kind == MCGB_SRC_ISOTROPIC_POINT) {
        /* IsotropicPoint.mcsim_launch, xopto/mcml/mcsource/point.py:76-128 */
        float sin_fi, cos_fi, R = 0.0f;
        v3 pos = {src->position[0], src->position[1], src->position[2]};
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rnd(x, a);
        float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        v3 d = {cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        v3 refracted = d;
        if (pos.z <= 0.0f) {
            float cc = c->layers[0].cos_critical_bottom;
            if (d.z > cc) {
                v3 normal = {0.0f, 0.0f, 1.0f};
                float n_sample = c->layers[1].n, n_medium = c->layers[0].n;
                refracted = refract3(d, normal, n_sample, n_medium);
                R = reflectance(n_medium, n_sample, d.z, cc);
                float t = -pos.z / d.z;
                pos.x += d.x * t;
                pos.y += d.y * t;
            } else {
                R = 1.0f;
            }
            pos.z = 0.0f;
        }
        s->dir = refracted;
        s->pos = pos;
        if (c->specular.kind != MCGB_DET_NONE)
            detector_deposit(mm, &c->specular, s->pos, d, R, 0.0f, accu, NULL);
        s->w = 1.0f - R;
        s->layer = src->layer_index;
    } else if (src->kind == MCGB_SRC_UNIFORM_RECTANGULAR ||
               src->kind == MCGB_SRC_LAMBERTIAN_RECTANGULAR ||
               src->kind == MCGB_SRC_UNIFORM_RECTANGULAR_LUT) {
        /* UniformRectangular / LambertianRectangular / UniformRectangularLut
           .mcsim_launch, xopto/mcml/mcsource/rectangular.py:85-140,363-413,
           600-650 */
        float sin_fi, cos_fi, sin_theta, cos_theta;
        s->pos.x = src->position[0] + (rnd(x, a) - 0.5f) * src->sigma[0];
        s->pos.y = src->position[1] + (rnd(x, a) - 0.5f) * src->sigma[1];
        s->pos.z = src->position[2];
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        if (src->kind == MCGB_SRC_UNIFORM_RECTANGULAR) {
            cos_theta = 1.0f - rnd(x, a) * (1.0f - src->angular);
            sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        } else if (src->kind == MCGB_SRC_UNIFORM_RECTANGULAR_LUT) {
            cos_theta = lut_rel(lut + src->lut_offset, src->lut_size, rnd(x, a), 0.0f);
            sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        } else {
            sin_theta = sqrtf(rnd(x, a)) * src->angular;
        }
        float n_layer = c->layers[src->layer_index].n;
        sin_theta = sin_theta / n_layer;
        cos_theta = sqrtf(1.0f - sin_theta * sin_theta);
        s->dir.x = cos_fi * sin_theta;
        s->dir.y = sin_fi * sin_theta;
        s->dir.z = cos_theta;
        s->w = 1.0f - reflectance_cos2(src->clip, n_layer, cos_theta);
        s->layer = src->layer_index;
    } else if (src->kind >= MCGB_SRC_UNIFORM_FIBER_NI) {
        mcml_launch_fiber(mm, c, lut, s, x, a, accu);
        s->layer = 1;
    } else {
        float cos_fi, sin_fi, r;
        v3 pt_src, pt_mc;
        r = sqrtf(-2.0f * m_log(mm, 1.0f - rnd(x, a)));
        r = fminf(r, src->clip);
        m_sincos(mm, 6.28318548f * rnd(x, a), &sin_fi, &cos_fi);
        pt_src.x = r * cos_fi * src->sigma[0];
        pt_src.y = r * sin_fi * src->sigma[1];
        pt_src.z = 0.0f;
        const float *T = src->transformation;
        /* mc_transform_fpv3, xopto/mcbase/kernel/mcbase.template.c:380-386 */
        pt_mc.x = T[0] * pt_src.x + T[1] * pt_src.y + T[2] * pt_src.z;
        pt_mc.y = T[3] * pt_src.x + T[4] * pt_src.y + T[5] * pt_src.z;
        pt_mc.z = T[6] * pt_src.x + T[7] * pt_src.y + T[8] * pt_src.z;
        float k = (0.0f - pt_mc.z) / src->direction[2];
        pt_mc.x += k * src->direction[0];
        pt_mc.y += k * src->direction[1];
        pt_mc.z = 0.0f;
        s->pos.x = src->position[0] + pt_mc.x;
        s->pos.y = src->position[1] + pt_mc.y;
        s->pos.z = 0.0f;
        s->dir.x = src->direction[0]; s->dir.y = src->direction[1]; s->dir.z = src->direction[2];
        s->layer = 1;
        s->w = 1.0f - src->reflectance;
        if (c->specular.kind != MCGB_DET_NONE) {
            v3 dir_in = {s->dir.x, s->dir.y, -s->dir.z};
            v3 normal = {0.0f, 0.0f, -1.0f};
            v3 d = refract3(dir_in, normal, c->layers[1].n, c->layers[0].n);
            detector_deposit(mm, &c->specular, s->pos, d, src->reflectance, 0.0f, accu, NULL);
        }
    }
}

/* mcsim_boundary (mcml), xopto/mcml/kernel/mcml.template.c:80-203 */
/* mc_transform_fpv3 of (x, y, 0), xopto/mcbase/kernel/mcbase.template.c:683-690 */
static inline void ml_transform_xy(const float *T, float x, float y, float *ox, float *oy) {
    *ox = T[0] * x + T[1] * y + T[2] * 0.0f;
    *oy = T[3] * x + T[4] * y + T[5] * 0.0f;
}

static int ml_fiber_hit(const float *T, float x, float y, float core_r2, float core_n,
                        float core_cc, float clad_r2, float clad_n, float clad_cc, float *n2,
                        float *cc) {
    float lx, ly;
    ml_transform_xy(T, x, y, &lx, &ly);
    float r2 = lx * lx + ly * ly;
    if (r2 <= clad_r2) {
        if (r2 <= core_r2) {
            *n2 = core_n;
            *cc = core_cc;
        } else {
            *n2 = clad_n;
            *cc = clad_cc;
        }
        return 1;
    }
    return 0;
}

/* Surface layout handlers: LambertianReflector (xopto/mcml/mcsurface/lambertian.py:70-106),
   LinearArray (probe/lineararray.py:167-239), SixAroundOne (probe/sixaroundone.py:158-262),
   FiberArray (probe/fiberarray.py:136-187).  Returns 1 when the packet continues with the
   boundary parameters n2, cc and 0 when the layout reflected it; the LinearArray probe tip
   is tested around the last fibre (the loop's final relative position), as in the reference. */
static int mcml_surface(int mm, const McgbSurface *sf, const float *lut, MlState *s, float *n2,
                        float *cc, uint64_t *x, uint32_t a) {
    const float *t = lut + sf->table_offset;
    float px = s->pos.x, py = s->pos.y;
    if (sf->kind == MCGB_SURFACE_LAMBERTIAN) {
        if (rnd(x, a) > t[1]) {
            float sin_fi, cos_fi;
            float sin_theta = sqrtf(rnd(x, a));
            float cos_theta = sqrtf(1.0f - sin_theta * sin_theta);
            m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
            float z = (float)fsign(-s->dir.z) * cos_theta;
            s->dir.x = cos_fi * sin_theta;
            s->dir.y = sin_fi * sin_theta;
            s->dir.z = z;
        } else {
            s->dir.z = -s->dir.z;
        }
        s->w = s->w * t[0];
        return 0;
    }
    if (sf->kind == MCGB_SURFACE_LINEAR_ARRAY) {
        float fx = t[11], fy = t[12], mx = 0.0f, my = 0.0f;
        for (uint32_t i = 0; i < sf->n_fibers; ++i) {
            mx = px - fx;
            my = py - fy;
            if (ml_fiber_hit(t, mx, my, t[15], t[16], t[17], t[18], t[19], t[20], n2, cc)) return 1;
            fx += t[13];
            fy += t[14];
        }
        float cx = px - t[9], cy = py - t[10];
        /* mc_transform_fpv2, xopto/mcbase/kernel/mcbase.template.c:675-680 */
        float ox = fabsf(t[23] * cx + t[24] * cy);
        float oy = fabsf(t[25] * cx + t[26] * cy);
        if (ox <= t[27] && oy < t[28]) {
            *n2 = t[29];
            *cc = t[30];
            return 1;
        }
        if (mx * mx + my * my <= t[21]) {
            s->dir.z = -s->dir.z;
            s->w = s->w * t[22];
            return 0;
        }
        return 1;
    }
    if (sf->kind == MCGB_SURFACE_SIX_AROUND_ONE) {
        float rx = px - t[9], ry = py - t[10];
        if (ml_fiber_hit(t, rx, ry, t[12], t[13], t[14], t[15], t[16], t[17], n2, cc)) return 1;
        if (ml_fiber_hit(t, fabsf(rx) - t[11], ry, t[12], t[13], t[14], t[15], t[16], t[17], n2, cc))
            return 1;
        if (ml_fiber_hit(t, fabsf(rx) - t[11] * 0.5f, fabsf(ry) - t[11] * 0.8660254037844386f, t[12],
                         t[13], t[14], t[15], t[16], t[17], n2, cc))
            return 1;
        float r2 = rx * rx + ry * ry;
        if (r2 <= t[18]) {
            *n2 = t[19];
            *cc = t[20];
            return 1;
        }
        if (r2 <= t[21]) {
            s->dir.z = -s->dir.z;
            s->w = s->w * t[22];
            return 0;
        }
        return 1;
    }
    for (uint32_t i = 0; i < sf->n_fibers; ++i) {
        const float *f = t + 4 + (size_t)i * MCGB_SURFACE_FIBER_FLOATS;
        if (ml_fiber_hit(f, px - f[9], py - f[10], f[14], f[15], f[16], f[11], f[12], f[13], n2, cc))
            return 1;
    }
    float dx = px - t[0], dy = py - t[1];
    if (dx * dx + dy * dy <= t[2]) {
        s->dir.z = -s->dir.z;
        s->w = s->w * t[3];
        return 0;
    }
    return 1;
}

static uint32_t mcml_boundary(int mm, const McgbMcmlConfig *c, const float *lut, MlState *s,
                              int32_t next, uint64_t *x, uint32_t a) {
    float cc, cos1, sin1, cos2, sin2, n_cos1, n_cos2, n2, n1_d_n2, R, Rs, Rp;
    const McgbLayer *cur = &c->layers[s->layer];
    const McgbLayer *nxt = &c->layers[s->layer + fsign(s->dir.z)];
    cc = (s->dir.z < 0.0f) ? cur->cos_critical_top : cur->cos_critical_bottom;
    n2 = nxt->n;
    /* surface layouts, xopto/mcml/kernel/mcml.template.c:104-124 */
    int layout = 0;
    int32_t last = (int32_t)c->num_layers - 1;
    const McgbSurface *sf = (next == 0) ? &c->surface_top : &c->surface_bottom;
    if ((next == 0 || next == last) && sf->kind != MCGB_SURFACE_NONE) {
        layout = 1;
        if (!mcml_surface(mm, sf, lut, s, &n2, &cc, x, a)) return EV_REFLECTION;
    }
    if (!layout && cur->n == n2) {
        s->layer = next;
        return EV_REFRACTION;
    }
    s->dir.z = -s->dir.z;
    cos1 = fabsf(s->dir.z);
    if (cos1 > cc) {
        if (cos1 > 1.0f) {
            R = (cur->n - n2) / (cur->n + n2);
            if (R * R < rnd(x, a)) {
                s->layer = next;
                s->dir.z = -s->dir.z;
                return EV_REFRACTION;
            }
            return EV_REFLECTION;
        }
        n1_d_n2 = cur->n / n2;
        sin1 = sqrtf(1.0f - cos1 * cos1);
        if (cos1 >= 1.0f) sin1 = 0.0f;
        sin2 = fminf(1.0f, n1_d_n2 * sin1);
        cos2 = sqrtf(1.0f - sin2 * sin2);
        n_cos1 = n1_d_n2 * cos1;
        n_cos2 = n1_d_n2 * cos2;
        Rs = (n_cos1 - cos2) / (n_cos1 + cos2);
        Rs *= Rs;
        Rp = (n_cos2 - cos1) / (n_cos2 + cos1);
        Rp *= Rp;
        R = 0.5f * (Rs + Rp);
        if (cos1 <= 0.0f || sin2 == 1.0f) R = 1.0f;
        if (R < rnd(x, a)) {
            s->layer = next;
            s->dir.x *= n1_d_n2;
            s->dir.y *= n1_d_n2;
            s->dir.z = -copysignf(cos2, s->dir.z);
            return EV_REFRACTION;
        }
    }
    return EV_REFLECTION;
}

/* Simulates the packets of one stream: McKernel (mcml),
   xopto/mcml/kernel/mcml.template.c:346-824.  Returns the number of
   interaction steps. */
static uint64_t mcml_stream(int mm, const McgbMcmlConfig *c, const float *lut,
                            uint64_t *rng_x, uint32_t a, uint64_t first,
                            uint64_t stride, uint64_t *accu, float *fbuf,
                            int32_t *ibuf) {
    const McgbRunOptions *o = &c->opt;
    uint64_t x = *rng_x, steps = 0;
    v3 src_pos = {c->source.position[0], c->source.position[1], c->source.position[2]};
    float rmax2 = o->rmax * o->rmax;
    int use_trace = c->trace.flags != MCGB_TRACE_NONE;
    for (uint64_t p = first; p < c->num_packets; p += stride) {
        MlState s;
        TraceState ts;
        memset(&s, 0, sizeof(s));
        ts.photon_index = p; ts.trace_count = 0; ts.events = 0;
        mcml_launch(mm, c, lut, &s, &x, a, accu);
        uint32_t events = EV_LAUNCH;
#define MO_TRACE_SNAPSHOT() do { ts.pos = s.pos; ts.dir = s.dir; ts.w = s.w; ts.opl = s.opl; \
                                 ts.events = events; } while (0)
        if (use_trace && (c->trace.flags & MCGB_TRACE_START)) {
            MO_TRACE_SNAPSHOT();
            trace_event(&c->trace, &ts, fbuf);
        }
        int done = 0;
        uint64_t packet_steps = 0;
        while (!done) {
            const McgbLayer *L = &c->layers[s.layer];
            float step, deposit;
            ++steps;
            if (o->method == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT)
                step = -m_log(mm, rnd(&x, a)) / L->mus;
            else
                step = -m_log(mm, rnd(&x, a)) * L->inv_mut;
            step = fminf(step, FLT_MAX);
            int32_t next = s.layer;
            if (s.pos.z + step * s.dir.z < L->top) {
                --next;
                if (fabsf(s.dir.z) != 0.0f) step = (L->top - s.pos.z) / s.dir.z;
            }
            if (s.pos.z + step * s.dir.z >= L->bottom) {
                ++next;
                if (fabsf(s.dir.z) != 0.0f) step = (L->bottom - s.pos.z) / s.dir.z;
            }
            s.pos.x = s.pos.x + s.dir.x * step;
            s.pos.y = s.pos.y + s.dir.y * step;
            s.pos.z = s.pos.z + s.dir.z * step;
            if (o->track_optical_pathlength) s.opl += L->n * step;
            if (s.layer < next) s.pos.z = L->bottom;
            if (s.layer > next) s.pos.z = L->top;

            if (o->method == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
                /* mcml.template.c:584-666 */
                float mua = L->mua;
                float fraction = 1.0f - m_exp(mm, -mua * step);
                deposit = fraction * s.w;
                s.w -= deposit;
                events |= EV_ABSORPTION;
                if (c->fluence.kind != MCGB_FLUENCE_NONE) {
                    float step_back = (mua != 0.0f)
                        ? step - (-m_log(mm, 1.0f - rnd(&x, a) * fraction)) / mua : 0.0f;
                    v3 dp = {s.pos.x - step_back * s.dir.x, s.pos.y - step_back * s.dir.y,
                             s.pos.z - step_back * s.dir.z};
                    fluence_deposit(&c->fluence, dp, deposit, L->mua, accu);
                }
                if (next != s.layer) {
                    events |= mcml_boundary(mm, c, lut, &s, next, &x, a) | EV_BOUNDARY_HIT;
                    if (!(s.layer > 0 && s.layer < (int32_t)c->num_layers - 1)) {
                        if (s.layer <= 0)
                            detector_deposit(mm, &c->top, s.pos, s.dir, s.w, s.opl, accu, lut);
                        else if (s.layer >= (int32_t)c->num_layers - 1)
                            detector_deposit(mm, &c->bottom, s.pos, s.dir, s.w, s.opl, accu, lut);
                        done = 1;
                    }
                } else {
                    float az, ct = pf_sample(mm, c->pf_kind, &L->pf, lut, &x, a, &az, &s.dir);
                    scatter_direction(mm, &s.dir, ct, az);
                    events |= EV_SCATTERING;
                }
                if (s.w < o->packet_weight_min) {
                    if (o->use_lottery) {
                        if (rnd(&x, a) > o->lottery_chance) done = 1;
                        else s.w = s.w / o->lottery_chance;
                    } else {
                        done = 1;
                    }
                }
            } else {
                if (next != s.layer) {
                    events |= mcml_boundary(mm, c, lut, &s, next, &x, a) | EV_BOUNDARY_HIT;
                    if (!(s.layer > 0 && s.layer < (int32_t)c->num_layers - 1)) {
                        if (s.layer <= 0)
                            detector_deposit(mm, &c->top, s.pos, s.dir, s.w, s.opl, accu, lut);
                        else if (s.layer >= (int32_t)c->num_layers - 1)
                            detector_deposit(mm, &c->bottom, s.pos, s.dir, s.w, s.opl, accu, lut);
                        done = 1;
                    }
                } else if (o->method == MCGB_METHOD_ALBEDO_REJECTION) {
                    /* mcml.template.c:705-721 */
                    if (rnd(&x, a) < L->mua_inv_mut) {
                        deposit = s.w;
                        done = 1;
                        s.w -= deposit;
                        events |= EV_ABSORPTION;
                        if (c->fluence.kind != MCGB_FLUENCE_NONE)
                            fluence_deposit(&c->fluence, s.pos, deposit, L->mua, accu);
                    } else {
                        float az, ct = pf_sample(mm, c->pf_kind, &L->pf, lut, &x, a, &az, &s.dir);
                        scatter_direction(mm, &s.dir, ct, az);
                        events |= EV_SCATTERING;
                    }
                } else {
                    /* albedo weight, mcml.template.c:722-753 */
                    deposit = s.w * L->mua_inv_mut;
                    s.w -= deposit;
                    events |= EV_ABSORPTION;
                    if (c->fluence.kind != MCGB_FLUENCE_NONE)
                        fluence_deposit(&c->fluence, s.pos, deposit, L->mua, accu);
                    float az, ct = pf_sample(mm, c->pf_kind, &L->pf, lut, &x, a, &az, &s.dir);
                    scatter_direction(mm, &s.dir, ct, az);
                    events |= EV_SCATTERING;
                    if (s.w < o->packet_weight_min) {
                        if (o->use_lottery) {
                            if (rnd(&x, a) > o->lottery_chance) done = 1;
                            else s.w = s.w / o->lottery_chance;
                        } else {
                            done = 1;
                        }
                    }
                }
            }
            /* rmax, mcml.template.c:759-763 */
            v3 d = {s.pos.x - src_pos.x, s.pos.y - src_pos.y, s.pos.z - src_pos.z};
            if (dot3(d, d) > rmax2) {
                done = 1;
                events |= EV_ESCAPED;
            }
            if (done) events |= EV_TERMINATED;
            if (use_trace) {
                if (c->trace.flags == MCGB_TRACE_ALL ||
                    ((c->trace.flags & MCGB_TRACE_END) && done)) {
                    MO_TRACE_SNAPSHOT();
                    trace_event(&c->trace, &ts, fbuf);
                }
            }
            events = 0;
            if (!done && o->max_steps_per_packet && ++packet_steps >= o->max_steps_per_packet)
                done = 1;
        }
        if (use_trace)
            ibuf[c->trace.count_offset + p] = (int32_t)ts.trace_count;
#undef MO_TRACE_SNAPSHOT
    }
    *rng_x = x;
    return steps;
}

/* ================================================================ mcvox */
typedef struct {
    v3 pos, dir;
    i3 vox;
    int32_t mat;
    float w, opl;
} MvState;

static inline int mv_valid(const McgbMcvoxConfig *c, i3 i) {
    return i.x >= 0 && i.x < c->shape[0] && i.y >= 0 && i.y < c->shape[1] &&
           i.z >= 0 && i.z < c->shape[2];
}
/* mcsim_flat_voxel_index, xopto/mcvox/kernel/mcvox.template.h:786-804 */
static inline int32_t mv_material_at(const McgbMcvoxConfig *c, const uint8_t *vox, i3 i) {
    uint64_t flat = ((uint64_t)i.z * (uint64_t)c->shape[1] + (uint64_t)i.y) *
                    (uint64_t)c->shape[0] + (uint64_t)i.x;
    return vox[flat];
}
/* mcsim_position_to_voxel_index, xopto/mcvox/kernel/mcvox.template.c:206-220 */
static inline i3 mv_index(const McgbMcvoxConfig *c, v3 p) {
    i3 r;
    r.x = cvt_int((p.x - c->top_left[0]) / c->voxel_size[0]);
    r.y = cvt_int((p.y - c->top_left[1]) / c->voxel_size[1]);
    r.z = cvt_int((p.z - c->top_left[2]) / c->voxel_size[2]);
    return r;
}

/* mcsim_sample_box_intersect, xopto/mcvox/kernel/mcvox.template.c:94-162 */
static int mv_box_intersect(const McgbMcvoxConfig *c, v3 pos, v3 dir, v3 *isec, v3 *normal) {
    float ix = (dir.x != 0.0f) ? 1.0f / dir.x : INFINITY;
    float iy = (dir.y != 0.0f) ? 1.0f / dir.y : INFINITY;
    float iz = (dir.z != 0.0f) ? 1.0f / dir.z : INFINITY;
    float t1 = (c->top_left[0] - pos.x) * ix;
    float t2 = (c->bottom_right[0] - pos.x) * ix;
    float t3 = (c->top_left[1] - pos.y) * iy;
    float t4 = (c->bottom_right[1] - pos.y) * iy;
    float t5 = (c->top_left[2] - pos.z) * iz;
    float t6 = (c->bottom_right[2] - pos.z) * iz;
    float txmin = fminf(t1, t2), txmax = fmaxf(t1, t2);
    float tymin = fminf(t3, t4), tymax = fmaxf(t3, t4);
    float tzmin = fminf(t5, t6), tzmax = fmaxf(t5, t6);
    float tmin = fmaxf(fmaxf(txmin, tymin), tzmin);
    float tmax = fminf(fminf(txmax, tymax), tzmax);
    if (tmin > tmax) return 0;
    normal->x = (float)(txmin >= tymin && txmin >= tzmin);
    normal->y = (float)((normal->x == 0.0f) && tymin >= tzmin);
    normal->z = (float)(normal->x == 0.0f && normal->y == 0.0f);
    normal->x *= (float)fsign(dir.x);
    normal->y *= (float)fsign(dir.y);
    normal->z *= (float)fsign(dir.z);
    float t = (tmin > 0.0f) ? tmin : tmax;
    isec->x = pos.x + t * dir.x;
    isec->y = pos.y + t * dir.y;
    isec->z = pos.z + t * dir.z;
    isec->x = fminf(fmaxf(isec->x, c->top_left[0]), c->bottom_right[0] - 1.1920929e-07f);
    isec->y = fminf(fmaxf(isec->y, c->top_left[1]), c->bottom_right[1] - 1.1920929e-07f);
    isec->z = fminf(fmaxf(isec->z, c->top_left[2]), c->bottom_right[2] - 1.1920929e-07f);
    return tmax >= tmin && tmax >= 0.0f;
}

/* mcsim_sample_box_contains, xopto/mcvox/kernel/mcvox.template.h:1227-1235 */
static int mv_contains(const McgbMcvoxConfig *c, v3 p) {
    return p.x >= c->top_left[0] && p.x < c->bottom_right[0] && p.y >= c->top_left[1] &&
           p.y < c->bottom_right[1] && p.z >= c->top_left[2] && p.z < c->bottom_right[2];
}

/* refractive index of the voxel at a point on the box surface
   (mcsim_position_to_voxel_index_safe + material lookup) */
static float mv_n_at_surface(const McgbMcvoxConfig *c, const McgbMaterial *mats,
                             const uint8_t *vox, v3 p) {
    i3 vi = mv_index(c, p);
    vi.x = clip_i(vi.x, 0, c->shape[0] - 1);
    vi.y = clip_i(vi.y, 0, c->shape[1] - 1);
    vi.z = clip_i(vi.z, 0, c->shape[2] - 1);
    return mats[mv_material_at(c, vox, vi)].n;
}

/* The beam entry into the voxel box of GaussianBeam.mcsim_launch
   (xopto/mcvox/mcsource/gaussianbeam.py:112-190) and UniformBeam.mcsim_launch
   (xopto/mcvox/mcsource/uniformbeam.py:104-186), from the beam point pt_mc. */
static void mv_beam_enter(int mm, const McgbMcvoxConfig *c, const McgbMaterial *mats,
                          const uint8_t *vox, MvState *s, v3 pt_mc, uint64_t *accu) {
    const McgbSource *src = &c->source;
    float specular_r;
    v3 direction = {src->direction[0], src->direction[1], src->direction[2]};
    if (mv_contains(c, pt_mc)) {
        direction.x = -direction.x; direction.y = -direction.y; direction.z = -direction.z;
    }
    v3 isec, normal;
    if (mv_box_intersect(c, pt_mc, direction, &isec, &normal)) {
        s->pos = isec;
        direction.x = -direction.x; direction.y = -direction.y; direction.z = -direction.z;
        normal.x = -normal.x; normal.y = -normal.y; normal.z = -normal.z;
        float n_outside = mats[0].n;
        float n_inside = mv_n_at_surface(c, mats, vox, s->pos);
        v3 refracted = direction;
        refract_safe3(direction, normal, n_outside, n_inside, &refracted);
        s->dir = refracted;
        specular_r = reflectance(n_outside, n_inside, dot3(normal, direction),
                                 cos_critical(n_outside, n_inside));
        if (c->specular.kind != MCGB_DET_NONE)
            detector_deposit(mm, &c->specular, s->pos, direction, specular_r, 0.0f, accu, NULL);
    } else {
        s->pos.x = c->top_left[0]; s->pos.y = c->top_left[1]; s->pos.z = c->top_left[2];
        s->dir.x = 0.0f; s->dir.y = 0.0f; s->dir.z = 1.0f;
        specular_r = 1.0f;
    }
    s->w = 1.0f - specular_r;
}

static inline v3 transform3(const float *T, v3 p) {
    /* mc_transform_fpv3, xopto/mcbase/kernel/mcbase.template.c:380-386 */
    v3 r;
    r.x = T[0] * p.x + T[1] * p.y + T[2] * p.z;
    r.y = T[3] * p.x + T[4] * p.y + T[5] * p.z;
    r.z = T[6] * p.x + T[7] * p.y + T[8] * p.z;
    return r;
}

/* mcsim_launch of the voxelized-medium sources: Line (xopto/mcvox/mcsource/line.py),
   GaussianBeam (gaussianbeam.py:112-190), UniformBeam (uniformbeam.py:104-186),
   IsotropicPoint (point.py:74-140), UniformFiber and LambertianFiber
   (fiber.py:257-352,603-700), IsotropicVoxel (voxel.py:78-107); then the voxel
   of the launch position (xopto/mcvox/kernel/mcvox.template.c:240-262). */
static void mcvox_launch(int mm, const McgbMcvoxConfig *c, const McgbMaterial *mats,
                         const uint8_t *vox, const float *lut, MvState *s, uint64_t *x,
                         uint32_t a, uint64_t *accu, v3 prev_pos) {
    const McgbSource *src = &c->source;
    const float *T = src->transformation;
    if (src->kind == MCGB_SRC_LINE) {
        /* xopto/mcvox/mcsource/line.py: position and directions are
           precomputed on the host by Line.cl_pack */
        s->w = 1.0f - src->reflectance;
        s->pos.x = src->position[0]; s->pos.y = src->position[1]; s->pos.z = src->position[2];
        s->dir.x = src->direction[0]; s->dir.y = src->direction[1]; s->dir.z = src->direction[2];
        if (c->specular.kind != MCGB_DET_NONE) {
            v3 d = {src->direction_reflected[0], src->direction_reflected[1],
                    src->direction_reflected[2]};
            detector_deposit(mm, &c->specular, s->pos, d, src->reflectance, 0.0f, accu, NULL);
        }
    } else if (src->kind == MCGB_SRC_GAUSSIAN_BEAM || src->kind == MCGB_SRC_UNIFORM_BEAM) {
        float cos_fi, sin_fi;
        v3 pt_src, pt_mc;
        if (src->kind == MCGB_SRC_GAUSSIAN_BEAM) {
            float r = sqrtf(-2.0f * m_log(mm, 1.0f - rnd(x, a)));
            r = fminf(r, src->clip);
            m_sincos(mm, 6.28318548f * rnd(x, a), &sin_fi, &cos_fi);
            pt_src.x = r * cos_fi * src->sigma[0];
            pt_src.y = r * sin_fi * src->sigma[1];
        } else {
            float rand_sqrt = sqrtf(rnd(x, a));
            float fi = 6.28318548f * rnd(x, a);
            m_sin_cos(mm, fi, &sin_fi, &cos_fi);
            pt_src.x = rand_sqrt * cos_fi * src->sigma[0];
            pt_src.y = rand_sqrt * sin_fi * src->sigma[1];
        }
        pt_src.z = 0.0f;
        pt_mc = transform3(T, pt_src);
        pt_mc.x += src->position[0];
        pt_mc.y += src->position[1];
        pt_mc.z += src->position[2];
        mv_beam_enter(mm, c, mats, vox, s, pt_mc, accu);
    } else if (src->kind == MCGB_SRC_ISOTROPIC_POINT) {
        /* Two quirks of the reference, restated: the refraction goes to a
           shadowing local variable, so the direction stays unrefracted
           (point.py:115-117); and mcsim_position_to_voxel_index reads the
           simulator's current position, not its argument
           (xopto/mcvox/kernel/mcvox.template.c:206-220), so the material
           that sets n_inside is the one at the previous packet's final
           position (prev_pos; the origin for a stream's first packet). */
        float sin_fi, cos_fi, specular_r = 0.0f;
        v3 pos = {src->position[0], src->position[1], src->position[2]};
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rnd(x, a);
        float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        v3 d = {cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        if (!mv_contains(c, pos)) {
            v3 isec, normal;
            if (mv_box_intersect(c, pos, d, &isec, &normal)) {
                pos = isec;
                float n_outside = mats[0].n;
                float n_inside = mv_n_at_surface(c, mats, vox, prev_pos);
                specular_r = reflectance(n_outside, n_inside, dot3(normal, d),
                                         cos_critical(n_outside, n_inside));
            } else {
                pos.x = c->top_left[0]; pos.y = c->top_left[1]; pos.z = c->top_left[2];
                specular_r = 1.0f;
            }
        }
        s->pos = pos;
        s->dir = d;
        if (c->specular.kind != MCGB_DET_NONE)
            detector_deposit(mm, &c->specular, s->pos, d, specular_r, 0.0f, accu, NULL);
        s->w = 1.0f - specular_r;
    } else if (src->kind == MCGB_SRC_UNIFORM_FIBER || src->kind == MCGB_SRC_LAMBERTIAN_FIBER ||
               src->kind == MCGB_SRC_UNIFORM_FIBER_LUT) {
        /* UniformFiberLut: cosine from the emission LUT,
           xopto/mcvox/mcsource/fiber.py:843-845 */
        float sin_fi, cos_fi, sin_theta, cos_theta, specular_r;
        float r = sqrtf(rnd(x, a)) * src->sigma[0];
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        v3 ps = {r * cos_fi, r * sin_fi, 0.0f};
        v3 pm = transform3(T, ps);
        pm.x += src->position[0];
        pm.y += src->position[1];
        pm.z += src->position[2];
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        if (src->kind == MCGB_SRC_LAMBERTIAN_FIBER) {
            sin_theta = sqrtf(rnd(x, a)) * src->sigma[1];
        } else {
            cos_theta = src->kind == MCGB_SRC_UNIFORM_FIBER_LUT
                            ? lut_rel(lut + src->lut_offset, src->lut_size, rnd(x, a), 0.0f)
                            : 1.0f - rnd(x, a) * (1.0f - src->sigma[1]);
            sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        }
        sin_theta = sin_theta / src->clip;
        cos_theta = sqrtf(1.0f - sin_theta * sin_theta);
        v3 pt = {cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        v3 packet_dir = transform3(T, pt);
        v3 source_dir = {src->direction[0], src->direction[1], src->direction[2]};
        if (mv_contains(c, pm)) {
            source_dir.x = -source_dir.x; source_dir.y = -source_dir.y; source_dir.z = -source_dir.z;
        }
        v3 refracted = packet_dir, isec, normal;
        if (mv_box_intersect(c, pm, source_dir, &isec, &normal)) {
            normal.x = -normal.x; normal.y = -normal.y; normal.z = -normal.z;
            s->pos = isec;
            float n_outside = src->clip;
            float n_inside = mv_n_at_surface(c, mats, vox, isec);
            refract_safe3(packet_dir, normal, n_outside, n_inside, &refracted);
            specular_r = reflectance(n_outside, n_inside, dot3(normal, packet_dir),
                                     cos_critical(n_outside, n_inside));
        } else {
            s->pos.x = c->top_left[0]; s->pos.y = c->top_left[1]; s->pos.z = c->top_left[2];
            specular_r = 1.0f;
        }
        s->dir = refracted;
        if (c->specular.kind != MCGB_DET_NONE)
            detector_deposit(mm, &c->specular, s->pos, packet_dir, specular_r, 0.0f, accu, NULL);
        s->w = 1.0f - specular_r;
    } else {
        /* IsotropicVoxel; IsotropicVoxels picks its voxel first,
           xopto/mcvox/mcsource/voxel.py:230-245 (mc_min of the int casts) */
        float vx = src->direction[0], vy = src->direction[1], vz = src->direction[2];
        s->w = 1.0f;
        if (src->kind == MCGB_SRC_ISOTROPIC_VOXELS) {
            int32_t n = (int32_t)src->lut_size;
            int32_t k = cvt_int(rnd(x, a) * (float)src->lut_size);
            if (k > n - 1) k = n - 1;
            const float *e = lut + src->lut_offset + (size_t)k * 4u;
            s->w = e[0];
            vx = e[1];
            vy = e[2];
            vz = e[3];
        }
        const float one_minus_eps = 1.0f - 1.1920929e-07f;
        s->pos.x = (vx + fminf(rnd(x, a), one_minus_eps)) * c->voxel_size[0] + c->top_left[0];
        s->pos.y = (vy + fminf(rnd(x, a), one_minus_eps)) * c->voxel_size[1] + c->top_left[1];
        s->pos.z = (vz + fminf(rnd(x, a), one_minus_eps)) * c->voxel_size[2] + c->top_left[2];
        float sin_fi, cos_fi;
        m_sincos(mm, rnd(x, a) * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rnd(x, a);
        float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        s->dir.x = cos_fi * sin_theta;
        s->dir.y = sin_fi * sin_theta;
        s->dir.z = cos_theta;
    }
    s->vox = mv_index(c, s->pos);
    s->mat = mv_valid(c, s->vox) ? mv_material_at(c, vox, s->vox) : 0;
}

/* mcsim_intersect, xopto/mcvox/kernel/mcvox.template.c:173-196 */
static float mv_intersect(const McgbMcvoxConfig *c, const MvState *s, v3 *d) {
    d->x = c->top_left[0] + (float)((s->dir.x >= 0.0f) + s->vox.x) * c->voxel_size[0] - s->pos.x;
    d->y = c->top_left[1] + (float)((s->dir.y >= 0.0f) + s->vox.y) * c->voxel_size[1] - s->pos.y;
    d->z = c->top_left[2] + (float)((s->dir.z >= 0.0f) + s->vox.z) * c->voxel_size[2] - s->pos.z;
    d->x = (s->dir.x != 0.0f) ? d->x / s->dir.x : INFINITY;
    d->y = (s->dir.y != 0.0f) ? d->y / s->dir.y : INFINITY;
    d->z = (s->dir.z != 0.0f) ? d->z / s->dir.z : INFINITY;
    return fminf(d->x, fminf(d->y, d->z));
}

/* mcsim_boundary (mcvox), xopto/mcvox/kernel/mcvox.template.c:275-388 */
static uint32_t mv_boundary(const McgbMcvoxConfig *c, const McgbMaterial *mats,
                            const uint8_t *vox, MvState *s, v3 dist, uint64_t *x, uint32_t a) {
    i3 nrm, nv;
    nrm.x = (dist.x <= dist.y) && (dist.x <= dist.z);
    nrm.y = nrm.x ? 0 : ((dist.y <= dist.x) && (dist.y <= dist.z));
    nrm.z = !(nrm.x + nrm.y);
    nrm.x = s->dir.x < 0.0f ? -nrm.x : nrm.x;
    nrm.y = s->dir.y < 0.0f ? -nrm.y : nrm.y;
    nrm.z = s->dir.z < 0.0f ? -nrm.z : nrm.z;
    nv.x = s->vox.x + nrm.x; nv.y = s->vox.y + nrm.y; nv.z = s->vox.z + nrm.z;
    int escaping = !mv_valid(c, nv);
    int32_t next_mat = !escaping ? mv_material_at(c, vox, nv) : 0;
    if (s->mat == next_mat && !escaping) {
        s->vox = nv;
        return EV_REFRACTION;
    }
    float n1 = mats[s->mat].n, n2 = mats[next_mat].n;
    if (n1 == n2) {
        s->vox = nv;
        s->mat = next_mat;
        return EV_REFRACTION;
    }
    float cc = cos_critical(n1, n2);
    float cos1 = (float)nrm.x * s->dir.x + (float)nrm.y * s->dir.y + (float)nrm.z * s->dir.z;
    v3 fn = {(float)nrm.x, (float)nrm.y, (float)nrm.z};
    if (cos1 > cc) {
        float R = reflectance(n1, n2, cos1, cc);
        if (R < rnd(x, a)) {
            s->dir = refract3(s->dir, fn, n1, n2);
            s->vox = nv;
            s->mat = next_mat;
            return EV_REFRACTION;
        }
    }
    s->dir = reflect3(s->dir, fn);
    return EV_REFLECTION;
}

/* McKernel (mcvox), xopto/mcvox/kernel/mcvox.template.c:548-1048 */
static uint64_t mcvox_stream(int mm, const McgbMcvoxConfig *c, const McgbMaterial *mats,
                             const uint8_t *vox, const float *lut, uint64_t *rng_x,
                             uint32_t a, uint64_t first, uint64_t stride,
                             uint64_t *accu, float *fbuf, int32_t *ibuf) {
    const McgbRunOptions *o = &c->opt;
    uint64_t x = *rng_x, steps = 0;
    v3 src_pos = {c->source.position[0], c->source.position[1], c->source.position[2]};
    float rmax2 = o->rmax * o->rmax;
    int use_trace = c->trace.flags != MCGB_TRACE_NONE;
    v3 prev_pos = {0.0f, 0.0f, 0.0f};     /* the stream's state position before launch */
    for (uint64_t p = first; p < c->num_packets; p += stride) {
        MvState s;
        TraceState ts;
        memset(&s, 0, sizeof(s));
        ts.photon_index = p; ts.trace_count = 0; ts.events = 0;
        mcvox_launch(mm, c, mats, vox, lut, &s, &x, a, accu, prev_pos);
        uint32_t events = EV_LAUNCH;
#define MV_TRACE_SNAPSHOT() do { ts.pos = s.pos; ts.dir = s.dir; ts.w = s.w; ts.opl = s.opl; \
                                 ts.events = events; } while (0)
        if (use_trace && (c->trace.flags & MCGB_TRACE_START)) {
            MV_TRACE_SNAPSHOT();
            trace_event(&c->trace, &ts, fbuf);
        }
        int done = 0;
        uint64_t packet_steps = 0;
        while (!done) {
            const McgbMaterial *M = &mats[s.mat];
            float step, deposit, d, d_ok;
            v3 dist;
            ++steps;
            if (o->method == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT)
                step = -m_log(mm, rnd(&x, a)) / M->mus;
            else
                step = -m_log(mm, rnd(&x, a)) * M->inv_mut;
            step = fminf(step, FLT_MAX);
            d = mv_intersect(c, &s, &dist);
            d_ok = fminf(d, step);
            s.pos.x = s.pos.x + d_ok * s.dir.x;
            s.pos.y = s.pos.y + d_ok * s.dir.y;
            s.pos.z = s.pos.z + d_ok * s.dir.z;
            if (o->track_optical_pathlength) s.opl += M->n * d_ok;
            if (o->method == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
                float mua = M->mua;
                float fraction = 1.0f - m_exp(mm, -mua * d_ok);
                deposit = fraction * s.w;
                s.w -= deposit;
                events |= EV_ABSORPTION;
                if (c->fluence.kind != MCGB_FLUENCE_NONE) {
                    float step_back = (mua != 0.0f)
                        ? d_ok - (-m_log(mm, 1.0f - rnd(&x, a) * fraction)) / mua : 0.0f;
                    v3 dp = {s.pos.x - step_back * s.dir.x, s.pos.y - step_back * s.dir.y,
                             s.pos.z - step_back * s.dir.z};
                    fluence_deposit(&c->fluence, dp, deposit, M->mua, accu);
                }
                if (d < step) {
                    events |= mv_boundary(c, mats, vox, &s, dist, &x, a) | EV_BOUNDARY_HIT;
                    if (!mv_valid(c, s.vox)) {
                        if (s.vox.z < 0)
                            detector_deposit(mm, &c->top, s.pos, s.dir, s.w, s.opl, accu, lut);
                        else if (s.vox.z >= c->shape[2])
                            detector_deposit(mm, &c->bottom, s.pos, s.dir, s.w, s.opl, accu, lut);
                        done = 1;
                    }
                } else {
                    float az, ct = pf_sample(mm, c->pf_kind, &M->pf, lut, &x, a, &az, &s.dir);
                    scatter_direction(mm, &s.dir, ct, az);
                    events |= EV_SCATTERING;
                }
                if (s.w < o->packet_weight_min) {
                    if (o->use_lottery) {
                        if (rnd(&x, a) > o->lottery_chance) done = 1;
                        else s.w = s.w / o->lottery_chance;
                    } else {
                        done = 1;
                    }
                }
            } else {
                if (d < step) {
                    events |= mv_boundary(c, mats, vox, &s, dist, &x, a) | EV_BOUNDARY_HIT;
                    if (!mv_valid(c, s.vox)) {
                        if (s.vox.z < 0)
                            detector_deposit(mm, &c->top, s.pos, s.dir, s.w, s.opl, accu, lut);
                        else if (s.vox.z >= c->shape[2])
                            detector_deposit(mm, &c->bottom, s.pos, s.dir, s.w, s.opl, accu, lut);
                        done = 1;
                    }
                } else if (o->method == MCGB_METHOD_ALBEDO_REJECTION) {
                    if (rnd(&x, a) < M->mua_inv_mut) {
                        deposit = s.w;
                        s.w -= deposit;
                        events |= EV_ABSORPTION;
                        done = 1;
                        if (c->fluence.kind != MCGB_FLUENCE_NONE)
                            fluence_deposit(&c->fluence, s.pos, deposit, M->mua, accu);
                    } else {
                        float az, ct = pf_sample(mm, c->pf_kind, &M->pf, lut, &x, a, &az, &s.dir);
                        scatter_direction(mm, &s.dir, ct, az);
                        events |= EV_SCATTERING;
                    }
                } else {
                    deposit = s.w * M->mua_inv_mut;
                    s.w -= deposit;
                    events |= EV_ABSORPTION;
                    if (c->fluence.kind != MCGB_FLUENCE_NONE)
                        fluence_deposit(&c->fluence, s.pos, deposit, M->mua, accu);
                    float az, ct = pf_sample(mm, c->pf_kind, &M->pf, lut, &x, a, &az, &s.dir);
                    scatter_direction(mm, &s.dir, ct, az);
                    events |= EV_SCATTERING;
                    if (s.w < o->packet_weight_min) {
                        if (o->use_lottery) {
                            if (rnd(&x, a) > o->lottery_chance) done = 1;
                            else s.w = s.w / o->lottery_chance;
                        } else {
                            done = 1;
                        }
                    }
                }
            }
            /* mcvox.template.c:1004-1008 */
            v3 dd = {s.pos.x - src_pos.x, s.pos.y - src_pos.y, s.pos.z - src_pos.z};
            if (dot3(dd, dd) > rmax2 || s.w <= 0.0f) {
                done = 1;
                events |= EV_ESCAPED;
            }
            if (done) events |= EV_TERMINATED;
            if (use_trace) {
                if (c->trace.flags == MCGB_TRACE_ALL ||
                    ((c->trace.flags & MCGB_TRACE_END) && done)) {
                    MV_TRACE_SNAPSHOT();
                    trace_event(&c->trace, &ts, fbuf);
                }
            }
            events = 0;
            if (!done && o->max_steps_per_packet && ++packet_steps >= o->max_steps_per_packet)
                done = 1;
        }
        if (use_trace)
            ibuf[c->trace.count_offset + p] = (int32_t)ts.trace_count;
        prev_pos = s.pos;
#undef MV_TRACE_SNAPSHOT
    }
    *rng_x = x;
    return steps;
}

/* ====================================================== exported API */
/* Runs every stream t < num_streams with the static packet mapping.  With
   nthreads > 1 the streams run on an OpenMP pool, each thread tallying into
   a private copy of the accumulator that is summed at the end (integer sums,
   so the result equals the serial run).  Returns the interaction steps. */
#define MO_RUN_BODY(STREAM_CALL)                                                    \
    uint64_t steps = 0;                                                             \
    int64_t T = cfg->num_streams;                                                   \
    if (nthreads <= 1) {                                                            \
        for (int64_t t = 0; t < T; ++t) {                                           \
            uint64_t *acc = accu;                                                   \
            steps += STREAM_CALL;                                                   \
        }                                                                           \
        return steps;                                                               \
    }                                                                               \
    int failed = 0;                                                                 \
    _Pragma("omp parallel num_threads(nthreads) reduction(+:steps)")               \
    {                                                                               \
        uint64_t *acc = (uint64_t *)calloc(accu_size ? accu_size : 1, 8);           \
        if (!acc) {                                                                 \
            _Pragma("omp atomic write") failed = 1;                                 \
        } else {                                                                    \
            _Pragma("omp for schedule(dynamic, 4)")                                 \
            for (int64_t t = 0; t < T; ++t) steps += STREAM_CALL;                   \
            _Pragma("omp critical")                                                 \
            for (uint64_t i = 0; i < accu_size; ++i) accu[i] += acc[i];             \
            free(acc);                                                              \
        }                                                                           \
    }                                                                               \
    return failed ? 0 : steps;

/* DYNAMIC scheduling: packet p on the stream of (seed, packet_offset + p)
   with the multipliers rng_a[0 .. num_streams); rng_x is unused. */
#define MO_DYNAMIC_BODY(PACKET_CALL)                                                 \
    uint64_t steps = 0;                                                              \
    int64_t N = (int64_t)cfg->num_packets;                                           \
    _Pragma("omp parallel num_threads(nthreads > 0 ? nthreads : 1) reduction(+:steps)") \
    {                                                                                \
        uint64_t *acc = (uint64_t *)calloc(accu_size ? accu_size : 1, 8);            \
        _Pragma("omp for schedule(dynamic, 16)")                                     \
        for (int64_t p = 0; p < N; ++p) {                                            \
            uint64_t x;                                                              \
            uint32_t a;                                                              \
            br_packet_stream(cfg->opt.seed, 0u, cfg->opt.packet_offset + (uint64_t)p, \
                             rng_a, cfg->num_streams, &x, &a);                       \
            steps += PACKET_CALL;                                                    \
        }                                                                            \
        _Pragma("omp critical")                                                      \
        for (uint64_t i = 0; i < accu_size; ++i) accu[i] += acc[i];                  \
        free(acc);                                                                   \
    }                                                                                \
    return steps;

uint64_t mco_mcml_run(int math_mode, const McgbMcmlConfig *cfg, const float *lut,
                      uint64_t *rng_x, const uint32_t *rng_a, uint64_t *accu,
                      uint64_t accu_size, float *fbuf, int32_t *ibuf, int nthreads) {
    if (cfg->opt.scheduling == MCGB_SCHED_DYNAMIC) {
        MO_DYNAMIC_BODY(mcml_stream(math_mode, cfg, lut, &x, a, (uint64_t)p, (uint64_t)N, acc,
                                    fbuf, ibuf))
    }
    MO_RUN_BODY(mcml_stream(math_mode, cfg, lut, &rng_x[t], rng_a[t], (uint64_t)t,
                            (uint64_t)T, acc, fbuf, ibuf))
}

uint64_t mco_mcvox_run(int math_mode, const McgbMcvoxConfig *cfg,
                       const McgbMaterial *materials, const uint8_t *voxels,
                       const float *lut, uint64_t *rng_x, const uint32_t *rng_a,
                       uint64_t *accu, uint64_t accu_size, float *fbuf, int32_t *ibuf,
                       int nthreads) {
    if (cfg->opt.scheduling == MCGB_SCHED_DYNAMIC) {
        MO_DYNAMIC_BODY(mcvox_stream(math_mode, cfg, materials, voxels, lut, &x, a, (uint64_t)p,
                                     (uint64_t)N, acc, fbuf, ibuf))
    }
    MO_RUN_BODY(mcvox_stream(math_mode, cfg, materials, voxels, lut, &rng_x[t], rng_a[t],
                             (uint64_t)t, (uint64_t)T, acc, fbuf, ibuf))
}

/* Stream of uniform random numbers (RngKernel, mcbase.template.c:1640-1646). */
void mco_rng_dump(uint64_t x, uint32_t a, uint64_t n, float *out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = rnd(&x, a);
}

/* Elementary functions for accuracy tests of the portable math. */
float mco_pm_log(float x) { return pm_logf(x); }
float mco_pm_exp(float x) { return pm_expf(x); }
float mco_pm_pow(float x, float y) { return pm_powrf(x, y); }
float mco_pm_cbrt(float x) { return pm_cbrtf(x); }
void mco_pm_sincos(float x, float *s, float *c) { pm_sincosf(x, s, c); }

/* ---------------------------------------------------------------------------
 * Sampling volume of packet traces: the reference's SamplingVolume kernel
 * (xopto/mcbase/kernel/mcsv.template.c:236-421) for all packets in order.
 * Each packet's recorded path is walked voxel by voxel: sva_voxel (:59-66)
 * truncates the first event's position to a voxel index, which is then only
 * stepped (sva_next_voxel, :136-160); the length travelled in a voxel is
 * summed across events and deposited when the walk leaves the voxel or the
 * path ends (sva_deposit_weight, :198-202).  The "end weight" is the last
 * float of the last recorded event (:299), which is the optical path length
 * slot of the trace entry (xopto/mcbase/mctrace.py:564-576).  Casts to
 * integers saturate (negative -> 0), as device conversions do; a packet with
 * no events is skipped (the reference would read before its trace).
 * Returns the status bits (MCGB_STATUS_BAD_INDEX when a walk hit the
 * crossing limit).
 * ------------------------------------------------------------------------- */
typedef struct { float x, y, z, px, py, pz; } SvEv;

static void sv_get(const float *tr, int32_t i, SvEv *e) {
    const float *f = tr + (size_t)i * MCGB_TRACE_ENTRY_LEN;
    e->x = f[0]; e->y = f[1]; e->z = f[2];
    e->px = f[3]; e->py = f[4]; e->pz = f[5];
}

static float sv_dist(const SvEv *a, const SvEv *b) {
    float dx = a->x - b->x, dy = a->y - b->y, dz = a->z - b->z;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

/* sva_intersect, mcsv.template.c:97-120 */
static float sv_axis_distance(float corner, int32_t v, float size, float pos, float dir) {
    float d = corner + (float)((dir >= 0.0f) + v) * size - pos;
    return (dir != 0.0f) ? d / dir : INFINITY;
}

uint64_t mco_sampling_volume(const McgbSamplingVolume *sv, const float *trace,
                             const int32_t *counts, uint64_t *accu, uint64_t *total_weight) {
    uint64_t status = 0;
    const float k = (float)sv->k;
    for (uint64_t p = 0; p < sv->num_packets; ++p) {
        int32_t n = counts[p] < (int32_t)sv->max_events ? counts[p] : (int32_t)sv->max_events;
        if (n <= 0) continue;
        const float *tr = trace + p * (uint64_t)sv->max_events * MCGB_TRACE_ENTRY_LEN;
        float end_w = tr[(size_t)n * MCGB_TRACE_ENTRY_LEN - 1];
        *total_weight += cvt_uint(end_w * k + 0.5f);
        SvEv e1, e2;
        int32_t ev = 0;
        sv_get(tr, 0, &e1);
        sv_get(tr, n - 1 < 1 ? n - 1 : 1, &e2);
        float d12 = sv_dist(&e1, &e2);
        int32_t vx = cvt_int((e1.x - sv->top_left[0]) / sv->voxel_size[0]);
        int32_t vy = cvt_int((e1.y - sv->top_left[1]) / sv->voxel_size[1]);
        int32_t vz = cvt_int((e1.z - sv->top_left[2]) / sv->voxel_size[2]);
        float l_voxel = 0.0f;
        uint32_t crossings = 0;
        for (;;) {
            float dx = sv_axis_distance(sv->top_left[0], vx, sv->voxel_size[0], e1.x, e1.px);
            float dy = sv_axis_distance(sv->top_left[1], vy, sv->voxel_size[1], e1.y, e1.py);
            float dz = sv_axis_distance(sv->top_left[2], vz, sv->voxel_size[2], e1.z, e1.pz);
            float d_voxel = fminf(dz, fminf(dx, dy));
            float d_move = fminf(d_voxel, d12);
            l_voxel += d_move;
            int inside = vx >= 0 && vy >= 0 && vz >= 0 && (uint32_t)vx < sv->shape[0] &&
                         (uint32_t)vy < sv->shape[1] && (uint32_t)vz < sv->shape[2];
            uint64_t flat = inside ? ((uint64_t)vz * sv->shape[1] + (uint64_t)vy) * sv->shape[0] +
                                     (uint64_t)vx : 0;
            if (d_voxel < d12) {
                if (inside)
                    accu[sv->offset + flat] += cvt_uint(end_w * l_voxel * sv->multiplier * k + 0.5f);
                e1.x += e1.px * d_move;
                e1.y += e1.py * d_move;
                e1.z += e1.pz * d_move;
                d12 -= d_move;
                int32_t nx = (dx <= dy) && (dx <= dz);
                int32_t ny = nx ? 0 : ((dy <= dx) && (dy <= dz));
                int32_t nz = !(nx + ny);
                vx += e1.px < 0.0f ? -nx : nx;
                vy += e1.py < 0.0f ? -ny : ny;
                vz += e1.pz < 0.0f ? -nz : nz;
                l_voxel = 0.0f;
                if (++crossings >= MCGB_SV_MAX_CROSSINGS) {
                    status |= MCGB_STATUS_BAD_INDEX;
                    break;
                }
            } else {
                e1 = e2;
                ev += 1;
                if (ev < n - 1) {
                    sv_get(tr, ev + 1, &e2);
                    d12 = sv_dist(&e1, &e2);
                } else {
                    if (inside)
                        accu[sv->offset + flat] += cvt_uint(end_w * l_voxel * sv->multiplier * k + 0.5f);
                    break;
                }
            }
        }
    }
    return status;
}

int mco_sizeof(int kind) {
    switch (kind) {
        case 0: return (int)sizeof(McgbLayer);
        case 1: return (int)sizeof(McgbSource);
        case 2: return (int)sizeof(McgbDetector);
        case 3: return (int)sizeof(McgbFluence);
        case 4: return (int)sizeof(McgbTrace);
        case 5: return (int)sizeof(McgbMaterial);
        case 14: return (int)sizeof(McgbSamplingVolume);
        case 6: return (int)sizeof(McgbMcmlConfig);
        case 7: return (int)sizeof(McgbMcvoxConfig);
        case 8: return (int)sizeof(McgbBuffers);
        case 9: return (int)sizeof(McgbRunOptions);
        case 10: return (int)sizeof(McgbPf);
        default: return -1;
    }
}

/* ===================================================== batched engine */
/* Per-simulation configuration of the batched engine as an mcml run:
   three layers (above, sample, below), Henyey-Greenstein phase function,
   normally incident Line source, radial top detector at offset
   sim*num_bins.  Layer fields follow the layered packing
   (xopto/mcml/mclayer/layer.py:304-354,944-1007) evaluated in double from
   the float simulation parameters. */
static double cc_d(double n1, double n2) { return n1 > n2 ? sqrt(1.0 - (n2 / n1) * (n2 / n1)) : 0.0; }

static void batch_sim_config(const McgbBatchConfig *bc, const McgbBatchSim *m, uint32_t sim,
                             McgbMcmlConfig *c) {
    memset(c, 0, sizeof(*c));
    c->num_packets = 1;
    c->num_streams = 1;
    c->pf_kind = MCGB_PF_HG;
    c->num_layers = 3;
    c->opt.method = MCGB_METHOD_ALBEDO_WEIGHT;
    c->opt.use_lottery = 1;
    c->opt.packet_weight_min = 1e-4f;
    c->opt.lottery_chance = 0.1f;
    c->opt.rmax = bc->rmax;
    double mua = m->mua, mus = m->mus, mut = mua + mus;
    McgbLayer *L = c->layers;
    L[0].top = -INFINITY; L[0].bottom = 0.0f; L[0].thickness = INFINITY;
    L[0].n = m->n_above; L[0].inv_mut = INFINITY; L[0].mua_inv_mut = 1.0f;
    L[0].cos_critical_bottom = (float)cc_d(m->n_above, m->n);
    L[1].top = 0.0f; L[1].bottom = m->thickness; L[1].thickness = m->thickness;
    L[1].n = m->n; L[1].mua = m->mua; L[1].mus = m->mus;
    L[1].inv_mut = mut > 0.0 ? (float)(1.0 / mut) : INFINITY;
    L[1].mua_inv_mut = mus == 0.0 ? 1.0f : (float)(mua * (mut > 0.0 ? 1.0 / mut : 0.0));
    L[1].cos_critical_top = (float)cc_d(m->n, m->n_above);
    L[1].cos_critical_bottom = (float)cc_d(m->n, m->n_below);
    L[1].pf.p[0] = m->g;
    L[2].top = m->thickness; L[2].bottom = INFINITY; L[2].thickness = INFINITY;
    L[2].n = m->n_below; L[2].inv_mut = INFINITY; L[2].mua_inv_mut = 1.0f;
    L[2].cos_critical_top = (float)cc_d(m->n_below, m->n);
    double r = ((double)m->n_above - m->n) / ((double)m->n_above + m->n);
    c->source.kind = MCGB_SRC_LINE;
    c->source.direction[2] = 1.0f;
    c->source.direction_reflected[2] = -1.0f;
    c->source.reflectance = (float)(r * r);
    c->top.kind = MCGB_DET_RADIAL;
    c->top.direction[2] = 1.0f;
    c->top.r_min = 0.0f;
    c->top.inv_dr = bc->inv_dr;
    c->top.cos_min = 0.0f;
    c->top.n = bc->num_bins;
    c->top.offset = (uint64_t)sim * bc->num_bins;
}

/* Every packet k of simulation s on its own stream (batch_rng.h); returns
   the interaction steps.  tally has num_sims*num_bins entries. */
uint64_t mco_batched_run(int math_mode, const McgbBatchConfig *bc, const McgbBatchSim *sims,
                         const uint32_t *mult, uint64_t *tally, int nthreads) {
    uint64_t steps = 0;
    int64_t S = bc->num_sims;
    uint64_t nt = (uint64_t)bc->num_sims * bc->num_bins;
    (void)nt;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) reduction(+:steps)
    {
        uint64_t *acc = (uint64_t *)calloc(nt ? nt : 1, 8);
        McgbMcmlConfig *c = (McgbMcmlConfig *)malloc(sizeof(McgbMcmlConfig));
#pragma omp for schedule(dynamic, 1)
        for (int64_t s = 0; s < S; ++s) {
            batch_sim_config(bc, &sims[s], (uint32_t)s, c);
            for (uint64_t k = 0; k < sims[s].num_packets; ++k) {
                uint64_t x;
                uint32_t a;
                br_packet_stream(bc->seed, (uint32_t)s, k, mult, bc->num_multipliers, &x, &a);
                steps += mcml_stream(math_mode, c, NULL, &x, a, 0, 1, acc, NULL, NULL);
            }
        }
#pragma omp critical
        for (uint64_t i = 0; i < nt; ++i) tally[i] += acc[i];
        free(acc);
        free(c);
    }
    return steps;
}
