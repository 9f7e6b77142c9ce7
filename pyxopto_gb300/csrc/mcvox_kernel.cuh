/*
 * mcvox_kernel.cuh - photon-packet transport in a voxelized sample
 * (the GB300 counterpart of McKernel, xopto/mcvox/kernel/mcvox.template.c:548-1048).
 *
 * Same thread/stream mapping and run control as the layered kernel.  Each
 * step moves the packet by min(free path, distance to the current voxel's
 * wall).  Voxels are stored as one uint8 material index each (the reference
 * uses a 4-byte McVoxel, xopto/mcvox/mcgeometry/voxel.py:33-85), read through
 * the read-only data cache; the material table lives in shared memory.
 */
#pragma once
#include "mc_device.cuh"

namespace MCGB_NS {

/* Shared-memory record of one material. */
struct __align__(16) MvMaterial {
    float4 g0;    /* mus, mua, inv_mut, mua_inv_mut */
    float4 g1;    /* n, -, -, - */
    float4 pf0;   /* phase-function constants (pf_prepare) */
    float4 pf1;
};

struct MvSmem {
    MvMaterial materials[MCGB_MAX_MATERIALS];
};

struct MvGeom {
    float tl[3], br[3], vs[3];
    int sh[3];
};

static __device__ __forceinline__ bool mv_valid(const MvGeom &g, const i3 &i) {
    return i.x >= 0 && i.x < g.sh[0] && i.y >= 0 && i.y < g.sh[1] && i.z >= 0 && i.z < g.sh[2];
}
/* mcsim_flat_voxel_index, xopto/mcvox/kernel/mcvox.template.h:786-804 */
static __device__ __forceinline__ int mv_material_at(const MvGeom &g, const uint8_t *vox, const i3 &i) {
    uint64_t flat = ((uint64_t)i.z * (uint64_t)g.sh[1] + (uint64_t)i.y) * (uint64_t)g.sh[0] + (uint64_t)i.x;
    return __ldg(vox + flat);
}
/* mcsim_position_to_voxel_index, mcvox.template.c:206-220 */
static __device__ __forceinline__ i3 mv_index(const MvGeom &g, const f3 &p) {
    return i3{cvt_int(mc_div(p.x - g.tl[0], g.vs[0])), cvt_int(mc_div(p.y - g.tl[1], g.vs[1])),
              cvt_int(mc_div(p.z - g.tl[2], g.vs[2]))};
}

/* mcsim_sample_box_intersect, mcvox.template.c:94-162 */
static __device__ __forceinline__ int mv_box_intersect(const MvGeom &g, const f3 &pos, const f3 &dir,
                                                       f3 &isec, f3 &normal) {
    float ix = (dir.x != 0.0f) ? mc_div(1.0f, dir.x) : __int_as_float(0x7f800000);
    float iy = (dir.y != 0.0f) ? mc_div(1.0f, dir.y) : __int_as_float(0x7f800000);
    float iz = (dir.z != 0.0f) ? mc_div(1.0f, dir.z) : __int_as_float(0x7f800000);
    float t1 = (g.tl[0] - pos.x) * ix, t2 = (g.br[0] - pos.x) * ix;
    float t3 = (g.tl[1] - pos.y) * iy, t4 = (g.br[1] - pos.y) * iy;
    float t5 = (g.tl[2] - pos.z) * iz, t6 = (g.br[2] - pos.z) * iz;
    float txmin = fminf(t1, t2), txmax = fmaxf(t1, t2);
    float tymin = fminf(t3, t4), tymax = fmaxf(t3, t4);
    float tzmin = fminf(t5, t6), tzmax = fmaxf(t5, t6);
    float tmin = fmaxf(fmaxf(txmin, tymin), tzmin);
    float tmax = fminf(fminf(txmax, tymax), tzmax);
    if (tmin > tmax) return 0;
    normal.x = (float)(txmin >= tymin && txmin >= tzmin);
    normal.y = (float)((normal.x == 0.0f) && tymin >= tzmin);
    normal.z = (float)(normal.x == 0.0f && normal.y == 0.0f);
    normal.x *= (float)fsign(dir.x);
    normal.y *= (float)fsign(dir.y);
    normal.z *= (float)fsign(dir.z);
    float tt = (tmin > 0.0f) ? tmin : tmax;
    isec.x = pos.x + tt * dir.x;
    isec.y = pos.y + tt * dir.y;
    isec.z = pos.z + tt * dir.z;
    isec.x = fminf(fmaxf(isec.x, g.tl[0]), g.br[0] - 1.1920929e-07f);
    isec.y = fminf(fmaxf(isec.y, g.tl[1]), g.br[1] - 1.1920929e-07f);
    isec.z = fminf(fmaxf(isec.z, g.tl[2]), g.br[2] - 1.1920929e-07f);
    return tmax >= tmin && tmax >= 0.0f;
}

/* Line launch (xopto/mcvox/mcsource/line.py) and GaussianBeam launch
   (xopto/mcvox/mcsource/gaussianbeam.py:112-190), then the voxel index of
   the launch position (mcvox.template.c:240-262). */
static __device__ __forceinline__ void mcvox_launch(const McgbMcvoxConfig &c, const MvGeom &g,
                                                    const MvMaterial *M, const uint8_t *vox,
                                                    Rng &rng, f3 &pos, f3 &dir, float &w, i3 &vi,
                                                    int &mat, uint64_t *accu) {
    const McgbSource &src = c.source;
    if (src.kind == MCGB_SRC_LINE) {
        w = 1.0f - src.reflectance;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 d{src.direction_reflected[0], src.direction_reflected[1], src.direction_reflected[2]};
            detector_deposit(c.specular, pos, d, src.reflectance, accu);
        }
    } else {
        float sin_fi, cos_fi, specular_r;
        float r = mc_sqrt(-2.0f * mc_log(1.0f - rng.next()));
        r = fminf(r, src.clip);
        mc_sincos(6.28318548f * rng.next(), &sin_fi, &cos_fi);
        f3 ps{r * cos_fi * src.sigma[0], r * sin_fi * src.sigma[1], 0.0f};
        const float *T = src.transformation;
        f3 pm{T[0] * ps.x + T[1] * ps.y + T[2] * ps.z,
              T[3] * ps.x + T[4] * ps.y + T[5] * ps.z,
              T[6] * ps.x + T[7] * ps.y + T[8] * ps.z};
        pm.x += src.position[0];
        pm.y += src.position[1];
        pm.z += src.position[2];
        f3 direction{src.direction[0], src.direction[1], src.direction[2]};
        if (pm.x >= g.tl[0] && pm.x < g.br[0] && pm.y >= g.tl[1] && pm.y < g.br[1] &&
            pm.z >= g.tl[2] && pm.z < g.br[2]) {
            direction = f3{-direction.x, -direction.y, -direction.z};
        }
        f3 isec, normal;
        if (mv_box_intersect(g, pm, direction, isec, normal)) {
            pos = isec;
            direction = f3{-direction.x, -direction.y, -direction.z};
            normal = f3{-normal.x, -normal.y, -normal.z};
            float n_outside = M[0].g1.x;
            i3 li = mv_index(g, pos);
            li.x = clip_i(li.x, 0, g.sh[0] - 1);
            li.y = clip_i(li.y, 0, g.sh[1] - 1);
            li.z = clip_i(li.z, 0, g.sh[2] - 1);
            float n_inside = M[mv_material_at(g, vox, li)].g1.x;
            f3 refracted = direction;
            refract_safe3(direction, normal, n_outside, n_inside, &refracted);
            dir = refracted;
            specular_r = reflectance(n_outside, n_inside, dot3(normal, direction),
                                     cos_critical(n_outside, n_inside));
            if (c.specular.kind != MCGB_DET_NONE)
                detector_deposit(c.specular, pos, direction, specular_r, accu);
        } else {
            pos = f3{g.tl[0], g.tl[1], g.tl[2]};
            dir = f3{0.0f, 0.0f, 1.0f};
            specular_r = 1.0f;
        }
        w = 1.0f - specular_r;
    }
    vi = mv_index(g, pos);
    mat = mv_valid(g, vi) ? mv_material_at(g, vox, vi) : 0;
}

/* mcsim_boundary (mcvox), mcvox.template.c:275-388 */
static __device__ __forceinline__ uint32_t mv_boundary(const MvGeom &g, const MvMaterial *M,
                                                       const uint8_t *vox, f3 &dir, i3 &vi,
                                                       int &mat, const f3 &dist, Rng &rng) {
    i3 nrm;
    nrm.x = (dist.x <= dist.y) && (dist.x <= dist.z);
    nrm.y = nrm.x ? 0 : ((dist.y <= dist.x) && (dist.y <= dist.z));
    nrm.z = !(nrm.x + nrm.y);
    nrm.x = dir.x < 0.0f ? -nrm.x : nrm.x;
    nrm.y = dir.y < 0.0f ? -nrm.y : nrm.y;
    nrm.z = dir.z < 0.0f ? -nrm.z : nrm.z;
    i3 nv{vi.x + nrm.x, vi.y + nrm.y, vi.z + nrm.z};
    bool escaping = !mv_valid(g, nv);
    int next_mat = !escaping ? mv_material_at(g, vox, nv) : 0;
    if (mat == next_mat && !escaping) {
        vi = nv;
        return MCGB_EV_REFRACTION;
    }
    float n1 = M[mat].g1.x, n2 = M[next_mat].g1.x;
    if (n1 == n2) {
        vi = nv;
        mat = next_mat;
        return MCGB_EV_REFRACTION;
    }
    float cc = cos_critical(n1, n2);
    float cos1 = (float)nrm.x * dir.x + (float)nrm.y * dir.y + (float)nrm.z * dir.z;
    f3 fn{(float)nrm.x, (float)nrm.y, (float)nrm.z};
    if (cos1 > cc) {
        float R = reflectance(n1, n2, cos1, cc);
        if (R < rng.next()) {
            dir = refract3(dir, fn, n1, n2);
            vi = nv;
            mat = next_mat;
            return MCGB_EV_REFRACTION;
        }
    }
    dir = reflect3(dir, fn);
    return MCGB_EV_REFLECTION;
}

template <int PF, int METHOD, bool FLU>
__global__ void __launch_bounds__(256)
mcvox_transport_kernel(const __grid_constant__ McgbMcvoxConfig c, const McgbBuffers b,
                       uint64_t deadline_ns, int lut_in_smem) {
    __shared__ MvSmem sm;
    extern __shared__ float s_lut[];
    for (uint32_t i = threadIdx.x; i < c.num_materials; i += blockDim.x) {
        const McgbMaterial &m = b.materials[i];
        MvMaterial h;
        h.g0 = make_float4(m.mus, m.mua, m.inv_mut, m.mua_inv_mut);
        h.g1 = make_float4(m.n, 0.0f, 0.0f, 0.0f);
        pf_prepare(PF, m.pf, h.pf0, h.pf1);
        sm.materials[i] = h;
    }
    if (lut_in_smem)
        for (uint64_t i = threadIdx.x; i < b.fp_lut_size; i += blockDim.x) s_lut[i] = b.fp_lut[i];
    __syncthreads();
    const float *lut = lut_in_smem ? s_lut : b.fp_lut;
    const MvMaterial *M = sm.materials;

    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.num_streams || t >= c.num_packets) return;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;

    MvGeom g;
    for (int k = 0; k < 3; ++k) {
        g.tl[k] = c.top_left[k]; g.br[k] = c.bottom_right[k];
        g.vs[k] = c.voxel_size[k]; g.sh[k] = c.shape[k];
    }
    const McgbRunOptions &o = c.opt;
    const uint64_t T = c.num_streams;
    const bool use_trace = c.trace.flags != MCGB_TRACE_NONE;
    const bool track_opl = o.track_optical_pathlength != 0;
    const float rmax2 = o.rmax * o.rmax;
    const bool use_rmax = rmax2 < __int_as_float(0x7f800000);
    const f3 src_pos{c.source.position[0], c.source.position[1], c.source.position[2]};
    const uint8_t *vox = b.voxels;
    uint64_t *accu = b.accumulator;

    Rng rng{b.rng_x[t], b.rng_a[t]};
    FluenceCache fcache{~0ull, 0};
    uint64_t steps = 0, packets = 0;
    uint32_t packet_steps = 0, iter = 0;
    uint32_t status = 0;

    uint64_t p = t;
    f3 pos, dir;
    i3 vi;
    int mat;
    float w, opl = 0.0f;
    uint32_t trace_count = 0, events = MCGB_EV_LAUNCH;
    mcvox_launch(c, g, M, vox, rng, pos, dir, w, vi, mat, accu);
    if (use_trace && (c.trace.flags & MCGB_TRACE_START))
        trace_event(c.trace, p, trace_count, events, pos, dir, w, opl, b.float_buffer);

    for (;;) {
        const float4 g0 = M[mat].g0;   /* mus, mua, inv_mut, mua_inv_mut */
        ++packet_steps;
        ++iter;
        float u = rng.next();
        float step = (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT)
                         ? mc_div(-mc_log(u), g0.x)
                         : -mc_log(u) * g0.z;
        step = fminf(step, FLT_MAX);
        /* mcsim_intersect, mcvox.template.c:173-196 */
        f3 dist;
        dist.x = g.tl[0] + (float)((dir.x >= 0.0f) + vi.x) * g.vs[0] - pos.x;
        dist.y = g.tl[1] + (float)((dir.y >= 0.0f) + vi.y) * g.vs[1] - pos.y;
        dist.z = g.tl[2] + (float)((dir.z >= 0.0f) + vi.z) * g.vs[2] - pos.z;
        dist.x = (dir.x != 0.0f) ? mc_div(dist.x, dir.x) : __int_as_float(0x7f800000);
        dist.y = (dir.y != 0.0f) ? mc_div(dist.y, dir.y) : __int_as_float(0x7f800000);
        dist.z = (dir.z != 0.0f) ? mc_div(dist.z, dir.z) : __int_as_float(0x7f800000);
        float d = fminf(dist.x, fminf(dist.y, dist.z));
        float d_ok = fminf(d, step);
        pos.x = pos.x + d_ok * dir.x;
        pos.y = pos.y + d_ok * dir.y;
        pos.z = pos.z + d_ok * dir.z;
        if (track_opl) opl += M[mat].g1.x * d_ok;

        bool done = false;
        if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
            float mua = g0.y;
            float fraction = 1.0f - mc_exp(-mua * d_ok);
            float deposit = fraction * w;
            w -= deposit;
            events |= MCGB_EV_ABSORPTION;
            if (FLU) {
                float step_back = (mua != 0.0f)
                                      ? d_ok - mc_div(-mc_log(1.0f - rng.next() * fraction), mua)
                                      : 0.0f;
                f3 dp{pos.x - step_back * dir.x, pos.y - step_back * dir.y, pos.z - step_back * dir.z};
                fluence_deposit(c.fluence, dp, deposit, mua, accu, fcache);
            }
            if (d < step) {
                events |= mv_boundary(g, M, vox, dir, vi, mat, dist, rng) | MCGB_EV_BOUNDARY_HIT;
                if (!mv_valid(g, vi)) {
                    if (vi.z < 0) detector_deposit(c.top, pos, dir, w, accu);
                    else if (vi.z >= g.sh[2]) detector_deposit(c.bottom, pos, dir, w, accu);
                    done = true;
                }
            } else {
                const MvMaterial &cm = M[mat];
                float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, lut, rng, &az);
                scatter_direction(dir, ct, az);
                events |= MCGB_EV_SCATTERING;
            }
            if (w < o.packet_weight_min) {
                if (o.use_lottery) {
                    if (rng.next() > o.lottery_chance) done = true;
                    else w = mc_div(w, o.lottery_chance);
                } else {
                    done = true;
                }
            }
        } else if (d < step) {
            events |= mv_boundary(g, M, vox, dir, vi, mat, dist, rng) | MCGB_EV_BOUNDARY_HIT;
            if (!mv_valid(g, vi)) {
                if (vi.z < 0) detector_deposit(c.top, pos, dir, w, accu);
                else if (vi.z >= g.sh[2]) detector_deposit(c.bottom, pos, dir, w, accu);
                done = true;
            }
        } else if (METHOD == MCGB_METHOD_ALBEDO_REJECTION) {
            if (rng.next() < g0.w) {
                float deposit = w;
                w -= deposit;
                events |= MCGB_EV_ABSORPTION;
                done = true;
                if (FLU) fluence_deposit(c.fluence, pos, deposit, g0.y, accu, fcache);
            } else {
                const MvMaterial &cm = M[mat];
                float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, lut, rng, &az);
                scatter_direction(dir, ct, az);
                events |= MCGB_EV_SCATTERING;
            }
        } else {
            float deposit = w * g0.w;
            w -= deposit;
            events |= MCGB_EV_ABSORPTION;
            if (FLU) fluence_deposit(c.fluence, pos, deposit, g0.y, accu, fcache);
            const MvMaterial &cm = M[mat];
            float az, ct = pf_sample<PF>(cm.pf0, cm.pf1, lut, rng, &az);
            scatter_direction(dir, ct, az);
            events |= MCGB_EV_SCATTERING;
            if (w < o.packet_weight_min) {
                if (o.use_lottery) {
                    if (rng.next() > o.lottery_chance) done = true;
                    else w = mc_div(w, o.lottery_chance);
                } else {
                    done = true;
                }
            }
        }
        /* mcvox.template.c:1004-1008 */
        bool escaped = w <= 0.0f;
        if (use_rmax) {
            f3 dd{pos.x - src_pos.x, pos.y - src_pos.y, pos.z - src_pos.z};
            escaped = escaped || dot3(dd, dd) > rmax2;
        }
        if (escaped) {
            done = true;
            events |= MCGB_EV_ESCAPED;
        }
        if (use_trace) {
            if (done) events |= MCGB_EV_TERMINATED;
            if (c.trace.flags == MCGB_TRACE_ALL || ((c.trace.flags & MCGB_TRACE_END) && done))
                trace_event(c.trace, p, trace_count, events, pos, dir, w, opl, b.float_buffer);
            events = 0;
        }
        if (!done && o.max_steps_per_packet && packet_steps >= o.max_steps_per_packet) {
            done = true;
            status |= MCGB_STATUS_STEP_LIMIT;
        }
        if (done) {
            ++packets;
            steps += packet_steps;
            packet_steps = 0;
            if (use_trace) b.int_buffer[c.trace.count_offset + p] = (int32_t)trace_count;
            p += T;
            if (p >= c.num_packets) break;
            trace_count = 0;
            opl = 0.0f;
            events = MCGB_EV_LAUNCH;
            mcvox_launch(c, g, M, vox, rng, pos, dir, w, vi, mat, accu);
            if (use_trace && (c.trace.flags & MCGB_TRACE_START))
                trace_event(c.trace, p, trace_count, events, pos, dir, w, opl, b.float_buffer);
        }
        if ((iter & 1023u) == 0) {
            if (globaltimer_ns() > t_deadline) { status |= MCGB_STATUS_TIMEOUT; break; }
            if (*(volatile uint64_t *)(b.counters + MCGB_CNT_ABORT)) { status |= MCGB_STATUS_ABORTED; break; }
        }
    }
    steps += packet_steps;
    if (FLU) fcache.flush(accu);
    b.rng_x[t] = rng.x;
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_STEPS), (unsigned long long)steps);
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_PACKETS), (unsigned long long)packets);
    atomicAdd((unsigned long long *)(b.counters + MCGB_CNT_THREADS), 1ull);
    if (status) atomicOr((unsigned long long *)(b.counters + MCGB_CNT_STATUS), (unsigned long long)status);
}

}  // namespace MCGB_NS
