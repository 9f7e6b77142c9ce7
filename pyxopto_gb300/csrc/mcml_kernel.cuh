/*
 * mcml_kernel.cuh - photon-packet transport in a stack of layers
 * (the GB300 counterpart of McKernel, xopto/mcml/kernel/mcml.template.c:346-824).
 *
 * One thread = one random-number stream.  Thread t simulates packets
 * t, t+T, t+2T, ... < N (T = num_streams); when a packet terminates the thread
 * launches its next packet inside the same loop iteration, so a warp keeps
 * all lanes busy until the lanes run out of packets.
 *
 * The layer table is rebuilt in shared memory as 16-byte records read with
 * vector loads (divergent per-lane layer indices hit distinct shared-memory
 * words instead of serialising on the constant cache); phase-function
 * constants are precomputed there once.  The kernel is specialised at compile
 * time on the phase function, the stepping method and whether a fluence grid
 * is tallied; traces and optical path length stay run-time options.
 *
 * Tallies are 64-bit integer atomics (detectors: one per escaping packet;
 * fluence: one per change of voxel through a per-thread cache).
 *
 * Run control: every 1024 loop iterations a thread compares %globaltimer with
 * its deadline and polls the host abort word; on expiry it sets a status
 * bit, stores its RNG state and leaves.  The kernel never waits on anything.
 */
#pragma once
#include "mc_device.cuh"
#include "batch_rng.h"

namespace MCGB_NS {

/* Shared-memory record of one layer. */
struct __align__(16) MlLayer {
    float4 g0;    /* top, bottom, step_factor(inv_mut), mua_inv_mut */
    float4 g1;    /* n, mua, mus, cos_critical_top */
    float4 pf0;   /* phase-function constants (pf_prepare) */
    float4 pf1;
    float4 g2;    /* cos_critical_bottom, -, -, - */
};

struct MlSmem {
    MlLayer layers[MCGB_MAX_LAYERS];
};

/* Fibre sources (xopto/mcml/mcsource/fiberni.py:246-290,485-534;
   fiber.py:267-330,576-640): a point uniform over the core; a direction
   uniform in solid angle within the acceptance cone (Uniform*) or with
   sin(theta) = sqrt(u)*NA (Lambertian*); the NI kinds refract the angle into
   the sample and weigh the launch with reflectance_cos2, the tilted kinds
   scale it by the core index, rotate both the point and the direction onto
   the fibre axis and weigh with the reflectance at the core/sample
   boundary.  The tilted kinds compare the launch point's z (0 on the
   surface) with the critical cosine before refracting, so the reference
   never refracts their direction; that is restated as is. */
static __device__ __forceinline__ void mcml_launch_fiber(const McgbMcmlConfig &c, const MlLayer *L,
                                                         const float *lut, Rng &rng, f3 &pos,
                                                         f3 &dir, float &w, uint64_t *accu) {
    const McgbSource &src = c.source;
    const bool from_lut = src.kind == MCGB_SRC_UNIFORM_FIBER_LUT_NI ||
                          src.kind == MCGB_SRC_UNIFORM_FIBER_LUT;
    const bool tilted = src.kind == MCGB_SRC_UNIFORM_FIBER || src.kind == MCGB_SRC_LAMBERTIAN_FIBER ||
                        src.kind == MCGB_SRC_UNIFORM_FIBER_LUT;
    const bool lambertian = src.kind == MCGB_SRC_LAMBERTIAN_FIBER_NI ||
                            src.kind == MCGB_SRC_LAMBERTIAN_FIBER;
    const float n_sample = L[1].g1.x, n_core = src.clip;
    const float *T = src.transformation;
    float sin_fi, cos_fi, sin_theta, cos_theta;
    float r = mc_sqrt(rng.next()) * src.sigma[0];
    mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
    if (tilted) {
        f3 ps{r * cos_fi, r * sin_fi, 0.0f};
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z, T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        float k = mc_div(0.0f - pm.z, src.direction[2]);
        pm.x += k * src.direction[0];
        pm.y += k * src.direction[1];
        pos = f3{src.position[0] + pm.x, src.position[1] + pm.y, 0.0f};
    } else {
        pos = f3{src.position[0] + r * cos_fi, src.position[1] + r * sin_fi, 0.0f};
    }
    mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
    if (lambertian) {
        sin_theta = mc_sqrt(rng.next()) * src.sigma[1];
    } else {
        cos_theta = from_lut ? lut_sample_rel(lut + src.lut_offset, src.lut_size, rng.next(), 0.0f)
                             : 1.0f - rng.next() * (1.0f - src.sigma[1]);
        sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
    }
    sin_theta = mc_div(sin_theta, tilted ? n_core : n_sample);
    cos_theta = mc_sqrt(1.0f - sin_theta * sin_theta);
    f3 pt{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
    float R;
    if (tilted) {
        f3 d{T[0] * pt.x + T[1] * pt.y + T[2] * pt.z, T[3] * pt.x + T[4] * pt.y + T[5] * pt.z,
             T[6] * pt.x + T[7] * pt.y + T[8] * pt.z};
        float cc = cos_critical(n_core, n_sample);
        dir = d;
        /* UniformFiberLut refracts into the sample (fiber.py:806-813);
           UniformFiber and LambertianFiber keep the direction in the core */
        if (from_lut && d.z > cc) dir = refract3(d, f3{0.0f, 0.0f, 1.0f}, n_core, n_sample);
        R = reflectance(n_core, n_sample, d.z, cc);
        if (c.specular.kind != MCGB_DET_NONE) detector_deposit(c.specular, pos, d, R, 0.0f, accu);
    } else {
        dir = pt;
        R = reflectance_cos2(n_core, n_sample, pt.z);
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 dir_in{dir.x, dir.y, -dir.z};
            f3 normal{0.0f, 0.0f, -1.0f};
            f3 d = refract3(dir_in, normal, n_sample, n_core);
            detector_deposit(c.specular, pos, d, R, 0.0f, accu);
        }
    }
    w = 1.0f - R;
}

/* GaussianBeam / UniformBeam / IsotropicPoint / fibre launch
   (xopto/mcml/mcsource/gaussianbeam.py:119-170, uniformbeam.py:107-146,
   point.py:76-128, fiberni.py, fiber.py). */
static __device__ __forceinline__ void mcml_launch_other(const McgbMcmlConfig &c, const MlLayer *L,
                                                         const float *lut, Rng &rng, f3 &pos,
                                                         f3 &dir, float &w, int &layer,
                                                         uint64_t *accu) {
    const McgbSource &src = c.source;
    if (src.kind == MCGB_SRC_UNIFORM_BEAM) {
        /* xopto/mcml/mcsource/uniformbeam.py:107-146 */
        float rand_sqrt = mc_sqrt(rng.next());
        float fi = 6.28318548f * rng.next();
        float sin_fi, cos_fi;
        mc_sincos(fi, &sin_fi, &cos_fi);
        f3 ps{rand_sqrt * cos_fi * src.sigma[0], rand_sqrt * sin_fi * src.sigma[1], 0.0f};
        const float *T = src.transformation;
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z, T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        float k = mc_div(0.0f - pm.z, src.direction[2]);
        pm.x += k * src.direction[0];
        pm.y += k * src.direction[1];
        pos = f3{src.position[0] + pm.x, src.position[1] + pm.y, 0.0f};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        w = 1.0f - src.reflectance;
        layer = 1;
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 dir_in{dir.x, dir.y, -dir.z};
            f3 normal{0.0f, 0.0f, -1.0f};
            f3 d = refract3(dir_in, normal, L[1].g1.x, L[0].g1.x);
            detector_deposit(c.specular, pos, d, src.reflectance, 0.0f, accu);
        }
    } else if (src.kind == MCGB_SRC_ISOTROPIC_POINT) {
        /* xopto/mcml/mcsource/point.py:76-128; the refraction into the
           sample passes (n_sample, n_medium) as (n1, n2), as the reference does */
        float sin_fi, cos_fi;
        float R = 0.0f;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        float cos_theta = 1.0f - 2.0f * rng.next();
        float sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        f3 d{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        dir = d;
        if (pos.z <= 0.0f) {
            float cc = L[0].g2.x;
            if (d.z > cc) {
                f3 normal{0.0f, 0.0f, 1.0f};
                float n_sample = L[1].g1.x, n_medium = L[0].g1.x;
                dir = refract3(d, normal, n_sample, n_medium);
                R = reflectance(n_medium, n_sample, d.z, cc);
                float t = mc_div(-pos.z, d.z);
                pos.x += d.x * t;
                pos.y += d.y * t;
            } else {
                R = 1.0f;
            }
            pos.z = 0.0f;
        }
        if (c.specular.kind != MCGB_DET_NONE) detector_deposit(c.specular, pos, d, R, 0.0f, accu);
        w = 1.0f - R;
        layer = src.layer_index;
    } else if (src.kind == MCGB_SRC_UNIFORM_RECTANGULAR || src.kind == MCGB_SRC_LAMBERTIAN_RECTANGULAR ||
               src.kind == MCGB_SRC_UNIFORM_RECTANGULAR_LUT) {
        /* xopto/mcml/mcsource/rectangular.py:85-140 (uniform in the cosine up
           to cos_min), 363-413 (Lambertian up to NA) and 600-650 (cosine from
           the emission LUT); the emission angle in air is refracted into the
           layer that holds the source */
        pos.x = src.position[0] + (rng.next() - 0.5f) * src.sigma[0];
        pos.y = src.position[1] + (rng.next() - 0.5f) * src.sigma[1];
        pos.z = src.position[2];
        float sin_fi, cos_fi, sin_theta, cos_theta;
        mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
        if (src.kind == MCGB_SRC_UNIFORM_RECTANGULAR) {
            cos_theta = 1.0f - rng.next() * (1.0f - src.angular);
            sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        } else if (src.kind == MCGB_SRC_UNIFORM_RECTANGULAR_LUT) {
            cos_theta = lut_sample_rel(lut + src.lut_offset, src.lut_size, rng.next(), 0.0f);
            sin_theta = mc_sqrt(1.0f - cos_theta * cos_theta);
        } else {
            sin_theta = mc_sqrt(rng.next()) * src.angular;
        }
        float n_layer = L[src.layer_index].g1.x;
        sin_theta = mc_div(sin_theta, n_layer);
        cos_theta = mc_sqrt(1.0f - sin_theta * sin_theta);
        dir = f3{cos_fi * sin_theta, sin_fi * sin_theta, cos_theta};
        w = 1.0f - reflectance_cos2(src.clip, n_layer, cos_theta);
        layer = src.layer_index;
    } else if (src.kind >= MCGB_SRC_UNIFORM_FIBER_NI) {
        mcml_launch_fiber(c, L, lut, rng, pos, dir, w, accu);
        layer = 1;
    } else {
        float sin_fi, cos_fi;
        float r = mc_sqrt(-2.0f * mc_log(1.0f - rng.next()));
        r = fminf(r, src.clip);
        mc_sincos(6.28318548f * rng.next(), &sin_fi, &cos_fi);
        f3 ps{r * cos_fi * src.sigma[0], r * sin_fi * src.sigma[1], 0.0f};
        const float *T = src.transformation;
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z,
              T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        float k = mc_div(0.0f - pm.z, src.direction[2]);
        pm.x += k * src.direction[0];
        pm.y += k * src.direction[1];
        pos = f3{src.position[0] + pm.x, src.position[1] + pm.y, 0.0f};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        layer = 1;
        w = 1.0f - src.reflectance;
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 dir_in{dir.x, dir.y, -dir.z};
            f3 normal{0.0f, 0.0f, -1.0f};
            f3 d = refract3(dir_in, normal, L[1].g1.x, L[0].g1.x);
            detector_deposit(c.specular, pos, d, src.reflectance, 0.0f, accu);
        }
    }
}

/* Packet launch: Line (xopto/mcml/mcsource/line.py:95-108) or any other
   source (mcml_launch_other).  SIMPLE kernels are compiled for the Line
   source only, which keeps the packet loop compact; everything stays inline
   (an out-of-line call measured slower). */
template <bool SIMPLE>
static __device__ __forceinline__ void mcml_launch(const McgbMcmlConfig &c, const MlLayer *L,
                                                   const float *lut, Rng &rng, f3 &pos, f3 &dir,
                                                   float &w, int &layer, uint64_t *accu) {
    const McgbSource &src = c.source;
    if (SIMPLE || src.kind == MCGB_SRC_LINE) {
        w = 1.0f - src.reflectance;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 d{src.direction_reflected[0], src.direction_reflected[1], src.direction_reflected[2]};
            detector_deposit(c.specular, pos, d, src.reflectance, 0.0f, accu);
        }
        layer = 1;
    } else {
        mcml_launch_other(c, L, lut, rng, pos, dir, w, layer, accu);
    }
}

/* 3x3 transformation of a point with z = 0 (mc_transform_fpv3,
   xopto/mcbase/kernel/mcbase.template.c:683-690; the z term is kept so the
   float operations match). */
static __device__ __forceinline__ float2 ml_transform_xy(const float *T, float x, float y) {
    return make_float2(T[0] * x + T[1] * y + T[2] * 0.0f, T[3] * x + T[4] * y + T[5] * 0.0f);
}

/* One fibre of a probe layout: core or cladding under the point (x, y)
   relative to the fibre centre, in the fibre's transformed frame. */
static __device__ __forceinline__ bool ml_fiber_hit(const float *T, float x, float y, float core_r2,
                                                    float core_n, float core_cc, float clad_r2,
                                                    float clad_n, float clad_cc, float &n2, float &cc,
                                                    float *r2_out = nullptr) {
    float2 lp = ml_transform_xy(T, x, y);
    float r2 = lp.x * lp.x + lp.y * lp.y;
    if (r2_out) *r2_out = r2;
    if (r2 <= clad_r2) {
        if (r2 <= core_r2) {
            n2 = core_n;
            cc = core_cc;
        } else {
            n2 = clad_n;
            cc = clad_cc;
        }
        return true;
    }
    return false;
}

/* Surface layout handler (mcsim_top/bottom_surface_layout_handler):
   LambertianReflector (xopto/mcml/mcsurface/lambertian.py:70-106),
   LinearArray (probe/lineararray.py:167-239), SixAroundOne
   (probe/sixaroundone.py:158-262) and FiberArray (probe/fiberarray.py:
   136-187).  Returns true when the packet continues with the boundary
   parameters n2, cc (possibly changed), false when the layout reflected it.
   As in the reference, the LinearArray probe tip is tested around the last
   fibre of the array (the loop's final relative position). */
static __device__ __forceinline__ bool mcml_surface(const McgbSurface &sf, const float *lut, f3 &dir,
                                                    float &w, float px, float py, float &n2,
                                                    float &cc, Rng &rng) {
    const float *t = lut + sf.table_offset;
    if (sf.kind == MCGB_SURFACE_LAMBERTIAN) {
        if (rng.next() > t[1]) {
            float sin_fi, cos_fi;
            float sin_theta = mc_sqrt(rng.next());
            float cos_theta = mc_sqrt(1.0f - sin_theta * sin_theta);
            mc_sincos(rng.next() * 6.28318548f, &sin_fi, &cos_fi);
            float z = (float)fsign(-dir.z) * cos_theta;
            dir = f3{cos_fi * sin_theta, sin_fi * sin_theta, z};
        } else {
            dir.z = -dir.z;
        }
        w = w * t[0];
        return false;
    }
    if (sf.kind == MCGB_SURFACE_LINEAR_ARRAY) {
        float fx = t[11], fy = t[12], mx = 0.0f, my = 0.0f;
        for (uint32_t i = 0; i < sf.n_fibers; ++i) {
            mx = px - fx;
            my = py - fy;
            if (ml_fiber_hit(t, mx, my, t[15], t[16], t[17], t[18], t[19], t[20], n2, cc)) return true;
            fx += t[13];
            fy += t[14];
        }
        float cx = px - t[9], cy = py - t[10];
        float ox = fabsf(t[23] * cx + t[24] * cy);
        float oy = fabsf(t[25] * cx + t[26] * cy);
        if (ox <= t[27] && oy < t[28]) {
            n2 = t[29];
            cc = t[30];
            return true;
        }
        if (mx * mx + my * my <= t[21]) {
            dir.z = -dir.z;
            w = w * t[22];
            return false;
        }
        return true;
    }
    if (sf.kind == MCGB_SURFACE_SIX_AROUND_ONE) {
        float rx = px - t[9], ry = py - t[10];
        if (ml_fiber_hit(t, rx, ry, t[12], t[13], t[14], t[15], t[16], t[17], n2, cc)) return true;
        if (ml_fiber_hit(t, fabsf(rx) - t[11], ry, t[12], t[13], t[14], t[15], t[16], t[17], n2, cc))
            return true;
        if (ml_fiber_hit(t, fabsf(rx) - t[11] * 0.5f, fabsf(ry) - t[11] * 0.8660254037844386f, t[12],
                         t[13], t[14], t[15], t[16], t[17], n2, cc))
            return true;
        float r2 = rx * rx + ry * ry;
        if (r2 <= t[18]) {
            n2 = t[19];
            cc = t[20];
            return true;
        }
        if (r2 <= t[21]) {
            dir.z = -dir.z;
            w = w * t[22];
            return false;
        }
        return true;
    }
    /* FIBER_ARRAY */
    for (uint32_t i = 0; i < sf.n_fibers; ++i) {
        const float *f = t + 4 + (size_t)i * MCGB_SURFACE_FIBER_FLOATS;
        if (ml_fiber_hit(f, px - f[9], py - f[10], f[14], f[15], f[16], f[11], f[12], f[13], n2, cc))
            return true;
    }
    float dx = px - t[0], dy = py - t[1];
    if (dx * dx + dy * dy <= t[2]) {
        dir.z = -dir.z;
        w = w * t[3];
        return false;
    }
    return true;
}

/* Reflect or refract at a layer boundary with Fresnel's equations, the
   common part of mcsim_boundary (xopto/mcml/kernel/mcml.template.c:135-203). */
static __device__ __forceinline__ uint32_t mcml_fresnel(int &layer, int next, float n1, float n2,
                                                        float cc, f3 &dir, Rng &rng) {
    dir.z = -dir.z;
    float cos1 = fabsf(dir.z);
    if (cos1 > cc) {
        if (cos1 > 1.0f) {
            float R = mc_div(n1 - n2, n1 + n2);
            if (R * R < rng.next()) {
                layer = next;
                dir.z = -dir.z;
                return MCGB_EV_REFRACTION;
            }
            return MCGB_EV_REFLECTION;
        }
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
        float R = 0.5f * (Rs + Rp);
        if (cos1 <= 0.0f || sin2 == 1.0f) R = 1.0f;
        if (R < rng.next()) {
            layer = next;
            dir.x *= n1_d_n2;
            dir.y *= n1_d_n2;
            dir.z = -copysignf(cos2, dir.z);
            return MCGB_EV_REFRACTION;
        }
    }
    return MCGB_EV_REFLECTION;
}

/* mcsim_boundary (mcml), xopto/mcml/kernel/mcml.template.c:80-203.  With
   XTRA the top and bottom surface layouts get the boundary first
   (mcml.template.c:104-124); a layout that lets the packet continue also
   skips the matched-index shortcut, as in the reference. */
template <bool XTRA>
static __device__ __forceinline__ uint32_t mcml_boundary(const McgbMcmlConfig &c, const float *lut,
                                                         const MlLayer *L, int &layer, int next,
                                                         int last, const f3 &pos, f3 &dir, float &w,
                                                         Rng &rng) {
    float cc = (dir.z < 0.0f) ? L[layer].g1.w : L[layer].g2.x;
    float n1 = L[layer].g1.x;
    float n2 = L[layer + fsign(dir.z)].g1.x;
    bool layout = false;
    if (XTRA) {
        const McgbSurface &sf = (next == 0) ? c.surface_top : c.surface_bottom;
        if ((next == 0 || next == last) && sf.kind != MCGB_SURFACE_NONE) {
            layout = true;
            if (!mcml_surface(sf, lut, dir, w, pos.x, pos.y, n2, cc, rng)) return MCGB_EV_REFLECTION;
        }
    }
    if (!layout && n1 == n2) {
        layer = next;
        return MCGB_EV_REFRACTION;
    }
    return mcml_fresnel(layer, next, n1, n2, cc, dir, rng);
}

/* mcsim_boundary without surface layouts (the batched engine). */
static __device__ __forceinline__ uint32_t mcml_boundary(const MlLayer *L, int &layer, int next,
                                                         f3 &dir, Rng &rng) {
    float cc = (dir.z < 0.0f) ? L[layer].g1.w : L[layer].g2.x;
    float n1 = L[layer].g1.x;
    float n2 = L[layer + fsign(dir.z)].g1.x;
    if (n1 == n2) {
        layer = next;
        return MCGB_EV_REFRACTION;
    }
    return mcml_fresnel(layer, next, n1, n2, cc, dir, rng);
}

/* Per-thread constants of a run. */
struct MlCtx {
    const MlLayer *L;
    const float *lut;
    float rmax2;
    bool use_rmax, use_trace, track_opl;
    uint32_t max_steps;   /* per-packet step limit, 0xFFFFFFFF when unlimited */
    int last_layer;
    f3 src_pos;
};

/* State of the packet a thread is simulating. */
struct MlPacket {
    f3 pos, dir;
    float w, opl;
    int layer;
    uint32_t trace_count, events, steps;
    uint64_t p;          /* packet number (trace slot) */
};

static __device__ __forceinline__ MlCtx mcml_ctx(const McgbMcmlConfig &c, const MlLayer *L,
                                                 const float *lut) {
    MlCtx x;
    x.L = L;
    x.lut = lut;
    x.rmax2 = c.opt.rmax * c.opt.rmax;
    /* dist2 > inf is never true: skip the test for an infinite rmax */
    x.use_rmax = x.rmax2 < __int_as_float(0x7f800000);
    x.use_trace = c.trace.flags != MCGB_TRACE_NONE;
    x.track_opl = c.opt.track_optical_pathlength != 0;
    x.max_steps = (c.opt.max_steps_per_packet == 0 || c.opt.max_steps_per_packet > 0xFFFFFFFFull)
                      ? 0xFFFFFFFFu : (uint32_t)c.opt.max_steps_per_packet;
    x.last_layer = (int)c.num_layers - 1;
    x.src_pos = f3{c.source.position[0], c.source.position[1], c.source.position[2]};
    return x;
}

template <bool SIMPLE>
static __device__ __forceinline__ void mcml_begin(const McgbMcmlConfig &c, const McgbBuffers &b,
                                                  const MlCtx &x, MlPacket &s, Rng &rng, uint64_t p) {
    s.p = p;
    s.opl = 0.0f;
    s.trace_count = 0;
    s.steps = 0;
    s.events = MCGB_EV_LAUNCH;
    mcml_launch<SIMPLE>(c, x.L, x.lut, rng, s.pos, s.dir, s.w, s.layer, b.accumulator);
    if (x.use_trace && (c.trace.flags & MCGB_TRACE_START))
        trace_event(c.trace, s.p, s.trace_count, s.events, s.pos, s.dir, s.w, s.opl, b.float_buffer);
}

static __device__ __forceinline__ void mcml_end(const McgbMcmlConfig &c, const McgbBuffers &b,
                                                const MlCtx &x, const MlPacket &s) {
    if (x.use_trace) b.int_buffer[c.trace.count_offset + s.p] = (int32_t)s.trace_count;
}

/* One interaction step of a packet (the body of McKernel's while(!done)
   loop, xopto/mcml/kernel/mcml.template.c:525-814).  Returns true when the
   packet terminated.  XTRA = false compiles out the optional features the
   launcher routes to the XTRA kernels: trace, optical path length, step
   limit, surface layouts, fibre-probe detectors and the fluence-rate
   scaling.  RMAX = false compiles out the rmax test (the launcher takes the
   SIMPLE kernels only without rmax). */
template <int PF, int METHOD, bool FLU, bool XTRA, bool RMAX = true>
static __device__ __forceinline__ bool mcml_step(const McgbMcmlConfig &c, const McgbBuffers &b,
                                                 const MlCtx &x, MlPacket &s, Rng &rng,
                                                 FluenceCache &fcache, uint32_t &status) {
    const MlLayer *L = x.L;
    const McgbRunOptions &o = c.opt;
    uint64_t *accu = b.accumulator;
    const float4 g0 = L[s.layer].g0;   /* top, bottom, step factor, mua_inv_mut */
    ++s.steps;
    float u = rng.next();
    float step;
    if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT)
        step = mc_div(-mc_log(u), L[s.layer].g1.z);
    else
        step = sample_step(u, g0.z);
    step = fminf(step, FLT_MAX);
    int next = s.layer;
    if (s.pos.z + step * s.dir.z < g0.x) {
        --next;
        if (fabsf(s.dir.z) != 0.0f) step = mc_div(g0.x - s.pos.z, s.dir.z);
    }
    if (s.pos.z + step * s.dir.z >= g0.y) {
        ++next;
        if (fabsf(s.dir.z) != 0.0f) step = mc_div(g0.y - s.pos.z, s.dir.z);
    }
    s.pos.x = s.pos.x + s.dir.x * step;
    s.pos.y = s.pos.y + s.dir.y * step;
    s.pos.z = s.pos.z + s.dir.z * step;
    if (XTRA && x.track_opl) s.opl += L[s.layer].g1.x * step;
    if (s.layer < next) s.pos.z = g0.y;
    if (s.layer > next) s.pos.z = g0.x;

    bool done = false;
    if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
        /* mcml.template.c:584-666 */
        float mua = L[s.layer].g1.y;
        float fraction = 1.0f - mc_exp(-mua * step);
        float deposit = fraction * s.w;
        s.w -= deposit;
        if (XTRA) s.events |= MCGB_EV_ABSORPTION;
        if (FLU) {
            float step_back = (mua != 0.0f)
                                  ? step - mc_div(-mc_log(1.0f - rng.next() * fraction), mua)
                                  : 0.0f;
            f3 dp{s.pos.x - step_back * s.dir.x, s.pos.y - step_back * s.dir.y,
                  s.pos.z - step_back * s.dir.z};
            fluence_deposit<XTRA>(c.fluence, dp, deposit, mua, fcache);
        }
        if (next != s.layer) {
            { uint32_t ev = mcml_boundary<XTRA>(c, x.lut, L, s.layer, next, x.last_layer, s.pos, s.dir, s.w, rng); if (XTRA) s.events |= ev | MCGB_EV_BOUNDARY_HIT; }
            if (!(s.layer > 0 && s.layer < x.last_layer)) {
                if (s.layer <= 0) detector_deposit<XTRA>(c.top, s.pos, s.dir, s.w, s.opl, accu, x.lut);
                else detector_deposit<XTRA>(c.bottom, s.pos, s.dir, s.w, s.opl, accu, x.lut);
                done = true;
            }
        } else {
            const MlLayer &cl = L[s.layer];
            float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, x.lut, rng, &az, s.dir);
            scatter_direction(s.dir, ct, az);
            if (XTRA) s.events |= MCGB_EV_SCATTERING;
        }
        if (s.w < o.packet_weight_min) {
            if (o.use_lottery) {
                if (rng.next() > o.lottery_chance) done = true;
                else s.w = mc_div(s.w, o.lottery_chance);
            } else {
                done = true;
            }
        }
    } else if (next != s.layer) {
        { uint32_t ev = mcml_boundary<XTRA>(c, x.lut, L, s.layer, next, x.last_layer, s.pos, s.dir, s.w, rng); if (XTRA) s.events |= ev | MCGB_EV_BOUNDARY_HIT; }
        if (!(s.layer > 0 && s.layer < x.last_layer)) {
            if (s.layer <= 0) detector_deposit<XTRA>(c.top, s.pos, s.dir, s.w, s.opl, accu, x.lut);
            else detector_deposit<XTRA>(c.bottom, s.pos, s.dir, s.w, s.opl, accu, x.lut);
            done = true;
        }
    } else if (METHOD == MCGB_METHOD_ALBEDO_REJECTION) {
        /* mcml.template.c:705-721 */
        if (rng.next() < g0.w) {
            float deposit = s.w;
            done = true;
            s.w -= deposit;
            if (XTRA) s.events |= MCGB_EV_ABSORPTION;
            if (FLU) fluence_deposit<XTRA>(c.fluence, s.pos, deposit, L[s.layer].g1.y, fcache);
        } else {
            const MlLayer &cl = L[s.layer];
            float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, x.lut, rng, &az, s.dir);
            scatter_direction(s.dir, ct, az);
            if (XTRA) s.events |= MCGB_EV_SCATTERING;
        }
    } else {
        /* albedo weight, mcml.template.c:722-753 */
        float deposit = s.w * g0.w;
        s.w -= deposit;
        if (XTRA) s.events |= MCGB_EV_ABSORPTION;
        if (FLU) fluence_deposit<XTRA>(c.fluence, s.pos, deposit, L[s.layer].g1.y, fcache);
        const MlLayer &cl = L[s.layer];
        float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, x.lut, rng, &az, s.dir);
        scatter_direction(s.dir, ct, az);
        if (XTRA) s.events |= MCGB_EV_SCATTERING;
        if (s.w < o.packet_weight_min) {
            if (o.use_lottery) {
                if (rng.next() > o.lottery_chance) done = true;
                else s.w = mc_div(s.w, o.lottery_chance);
            } else {
                done = true;
            }
        }
    }
    /* rmax, mcml.template.c:759-763 */
    if (RMAX && x.use_rmax) {
        f3 d{s.pos.x - x.src_pos.x, s.pos.y - x.src_pos.y, s.pos.z - x.src_pos.z};
        if (dot3(d, d) > x.rmax2) {
            done = true;
            if (XTRA) s.events |= MCGB_EV_ESCAPED;
        }
    }
    if (XTRA && x.use_trace) {
        if (done) s.events |= MCGB_EV_TERMINATED;
        if (c.trace.flags == MCGB_TRACE_ALL || ((c.trace.flags & MCGB_TRACE_END) && done))
            trace_event(c.trace, s.p, s.trace_count, s.events, s.pos, s.dir, s.w, s.opl, b.float_buffer);
        s.events = 0;
    }
    if (XTRA && !done && s.steps >= x.max_steps) {
        done = true;
        status |= MCGB_STATUS_STEP_LIMIT;
    }
    return done;
}

/* Shared-memory tables of one block. */
template <int PF>
static __device__ __forceinline__ const float *mcml_stage(const McgbMcmlConfig &c, const McgbBuffers &b,
                                                          MlSmem &sm, float *s_lut, int lut_in_smem) {
    for (uint32_t i = threadIdx.x; i < c.num_layers; i += blockDim.x) {
        const McgbLayer &l = c.layers[i];
        MlLayer h;
        h.g0 = make_float4(l.top, l.bottom, step_factor(l.inv_mut), l.mua_inv_mut);
        h.g1 = make_float4(l.n, l.mua, l.mus, l.cos_critical_top);
        h.g2 = make_float4(l.cos_critical_bottom, 0.0f, 0.0f, 0.0f);
        pf_prepare(PF, l.pf, h.pf0, h.pf1);
        sm.layers[i] = h;
    }
    if (lut_in_smem)
        for (uint64_t i = threadIdx.x; i < b.fp_lut_size; i += blockDim.x) s_lut[i] = b.fp_lut[i];
    __syncthreads();
    return lut_in_smem ? s_lut : b.fp_lut;
}

static __device__ __forceinline__ void mc_finish(const McgbBuffers &b, uint64_t steps, uint64_t packets,
                                                 uint32_t status, bool count_thread) {
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_STEPS), (unsigned long long)steps);
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_PACKETS), (unsigned long long)packets);
    if (count_thread) atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_THREADS), 1ull);
    if (status) atomicOr((unsigned long long *)(b.counters + MCGB_CNT_STATUS), (unsigned long long)status);
}

/* STATIC scheduling: thread t owns stream t and packets t, t+T, ... */
template <int PF, int METHOD, bool FLU>
__global__ void __launch_bounds__(256)
mcml_transport_kernel(const __grid_constant__ McgbMcmlConfig c, const McgbBuffers b,
                      uint64_t deadline_ns, int lut_in_smem, uint32_t packets_per_item) {
    __shared__ MlSmem sm;
    extern __shared__ float s_lut[];
    const float *lut = mcml_stage<PF>(c, b, sm, s_lut, lut_in_smem);
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.num_streams || t >= c.num_packets) return;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;
    const MlCtx x = mcml_ctx(c, sm.layers, lut);
    const uint64_t T = c.num_streams;
    Rng rng{b.rng_x[t], b.rng_a[t]};
    FluenceCache fcache = fluence_cache(c.fluence, b.accumulator);
    uint64_t steps = 0, packets = 0;
    uint32_t iter = 0, status = 0;
    MlPacket s;
    mcml_begin<false>(c, b, x, s, rng, t);
    for (;;) {
        if (mcml_step<PF, METHOD, FLU, true>(c, b, x, s, rng, fcache, status)) {
            ++packets;
            steps += s.steps;
            mcml_end(c, b, x, s);
            uint64_t p = s.p + T;
            if (p >= c.num_packets) {
                s.steps = 0;
                break;
            }
            mcml_begin<false>(c, b, x, s, rng, p);
        }
        if (((++iter) & 1023u) == 0) {
            if (globaltimer_ns() > t_deadline) { status |= MCGB_STATUS_TIMEOUT; break; }
            if (*(volatile uint64_t *)(b.counters + MCGB_CNT_ABORT)) { status |= MCGB_STATUS_ABORTED; break; }
        }
    }
    steps += s.steps;
    if (FLU) fcache.flush();
    b.rng_x[t] = rng.x;
    mc_finish(b, steps, packets, status, true);
}

#define MCGB_FULL_MASK 0xffffffffu

/* DYNAMIC scheduling: persistent warps refill idle lanes packet by packet
   from the queue counters[MCGB_CNT_QUEUE]; packet p runs on the stream of
   (seed, packet_offset + p). */
template <int PF, int METHOD, bool FLU, bool XTRA, bool SIMPLE>
__global__ void __launch_bounds__(128)
mcml_dynamic_kernel(const __grid_constant__ McgbMcmlConfig c, const McgbBuffers b,
                    uint64_t deadline_ns, int lut_in_smem, uint32_t packets_per_item) {
    __shared__ MlSmem sm;
    extern __shared__ float s_lut[];
    const float *lut = mcml_stage<PF>(c, b, sm, s_lut, lut_in_smem);
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;
    const MlCtx x = mcml_ctx(c, sm.layers, lut);
    const uint64_t N = c.num_packets;
    const uint64_t B = packets_per_item;
    unsigned long long *queue = (unsigned long long *)(b.counters + MCGB_CNT_QUEUE);
    uint64_t item_next = 0, item_end = 0;   /* warp-uniform */
    bool more = true, active = false;
    Rng rng{0ull, 1u};
    FluenceCache fcache = fluence_cache(c.fluence, b.accumulator);
    uint64_t steps = 0, packets = 0;
    uint32_t iter = 0, status = 0;
    MlPacket s;
    s.steps = 0;
    for (;;) {
        uint32_t need = __ballot_sync(MCGB_FULL_MASK, !active);
        while (need && more) {
            if (item_next >= item_end) {
                unsigned long long item = 0;
                if (lane == 0) item = atomicAdd(queue, 1ull);
                item = __shfl_sync(MCGB_FULL_MASK, item, 0);
                item_next = (uint64_t)item * B;
                if (item_next >= N) {
                    more = false;
                    break;
                }
                item_end = min(item_next + B, N);
            }
            uint32_t avail = (uint32_t)min(item_end - item_next, (uint64_t)32);
            uint32_t rank = __popc(need & ((1u << lane) - 1u));
            bool mine = ((need >> lane) & 1u) && rank < avail;
            if (mine) {
                uint64_t p = item_next + rank;
                uint64_t xs;
                uint32_t as;
                br_packet_stream(c.opt.seed, 0u, c.opt.packet_offset + p, b.rng_a, c.num_streams, &xs, &as);
                rng = Rng{xs, as};
                mcml_begin<SIMPLE>(c, b, x, s, rng, p);
                active = true;
            }
            uint32_t taken = __ballot_sync(MCGB_FULL_MASK, mine);
            item_next += __popc(taken);
            need &= ~taken;
        }
        if (!__any_sync(MCGB_FULL_MASK, active)) break;
        /* sixteen steps between refills; two steps per loop iteration give
           the scheduler both bodies (+0.9 % on the layered stack) */
#pragma unroll 2
        for (int k = 0; k < 16; ++k) {
            if (active && mcml_step<PF, METHOD, FLU, XTRA, XTRA || !SIMPLE>(c, b, x, s, rng, fcache, status)) {
                ++packets;
                steps += s.steps;
                s.steps = 0;
                mcml_end(c, b, x, s);
                active = false;
            }
        }
        iter += 16;
        if ((iter & 1023u) == 0) {
            uint32_t stop = 0;
            if (lane == 0) {
                if (globaltimer_ns() > t_deadline) stop = MCGB_STATUS_TIMEOUT;
                else if (*(volatile uint64_t *)(b.counters + MCGB_CNT_ABORT)) stop = MCGB_STATUS_ABORTED;
            }
            stop = __shfl_sync(MCGB_FULL_MASK, stop, 0);
            if (stop) {
                status |= stop;
                break;
            }
        }
    }
    steps += s.steps;
    if (FLU) fcache.flush();
    mc_finish(b, steps, packets, status, packets > 0);
}

}  // namespace MCGB_NS
