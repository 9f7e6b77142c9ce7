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

namespace MCGB_NS {

/* Shared-memory record of one layer. */
struct __align__(16) MlLayer {
    float4 g0;    /* top, bottom, inv_mut, mua_inv_mut */
    float4 g1;    /* n, mua, mus, cos_critical_top */
    float4 pf0;   /* phase-function constants (pf_prepare) */
    float4 pf1;
    float4 g2;    /* cos_critical_bottom, -, -, - */
};

struct MlSmem {
    MlLayer layers[MCGB_MAX_LAYERS];
};

/* Line / GaussianBeam launch (xopto/mcml/mcsource/line.py:95-108,
   gaussianbeam.py:119-170). */
static __device__ __forceinline__ void mcml_launch(const McgbMcmlConfig &c, const MlLayer *L,
                                                   Rng &rng, f3 &pos, f3 &dir, float &w,
                                                   int &layer, uint64_t *accu) {
    const McgbSource &src = c.source;
    if (src.kind == MCGB_SRC_LINE) {
        w = 1.0f - src.reflectance;
        pos = f3{src.position[0], src.position[1], src.position[2]};
        dir = f3{src.direction[0], src.direction[1], src.direction[2]};
        if (c.specular.kind != MCGB_DET_NONE) {
            f3 d{src.direction_reflected[0], src.direction_reflected[1], src.direction_reflected[2]};
            detector_deposit(c.specular, pos, d, src.reflectance, accu);
        }
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
            detector_deposit(c.specular, pos, d, src.reflectance, accu);
        }
    }
}

/* mcsim_boundary (mcml), xopto/mcml/kernel/mcml.template.c:80-203 */
static __device__ __forceinline__ uint32_t mcml_boundary(const MlLayer *L, int &layer, int next,
                                                         f3 &dir, Rng &rng) {
    float cc = (dir.z < 0.0f) ? L[layer].g1.w : L[layer].g2.x;
    float n1 = L[layer].g1.x;
    float n2 = L[layer + fsign(dir.z)].g1.x;
    if (n1 == n2) {
        layer = next;
        return MCGB_EV_REFRACTION;
    }
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

template <int PF, int METHOD, bool FLU>
__global__ void __launch_bounds__(256)
mcml_transport_kernel(const __grid_constant__ McgbMcmlConfig c, const McgbBuffers b,
                      uint64_t deadline_ns, int lut_in_smem) {
    __shared__ MlSmem sm;
    extern __shared__ float s_lut[];
    for (uint32_t i = threadIdx.x; i < c.num_layers; i += blockDim.x) {
        const McgbLayer &l = c.layers[i];
        MlLayer h;
        h.g0 = make_float4(l.top, l.bottom, l.inv_mut, l.mua_inv_mut);
        h.g1 = make_float4(l.n, l.mua, l.mus, l.cos_critical_top);
        h.g2 = make_float4(l.cos_critical_bottom, 0.0f, 0.0f, 0.0f);
        pf_prepare(PF, l.pf, h.pf0, h.pf1);
        sm.layers[i] = h;
    }
    if (lut_in_smem)
        for (uint64_t i = threadIdx.x; i < b.fp_lut_size; i += blockDim.x) s_lut[i] = b.fp_lut[i];
    __syncthreads();
    const float *lut = lut_in_smem ? s_lut : b.fp_lut;
    const MlLayer *L = sm.layers;

    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.num_streams || t >= c.num_packets) return;
    const uint64_t t_deadline = globaltimer_ns() + deadline_ns;

    const McgbRunOptions &o = c.opt;
    const uint64_t T = c.num_streams;
    const bool use_trace = c.trace.flags != MCGB_TRACE_NONE;
    const bool track_opl = o.track_optical_pathlength != 0;
    const float rmax2 = o.rmax * o.rmax;
    /* dist2 > inf is never true: skip the test for an infinite rmax */
    const bool use_rmax = rmax2 < __int_as_float(0x7f800000);
    const int last_layer = (int)c.num_layers - 1;
    const f3 src_pos{c.source.position[0], c.source.position[1], c.source.position[2]};
    uint64_t *accu = b.accumulator;

    Rng rng{b.rng_x[t], b.rng_a[t]};
    FluenceCache fcache{~0ull, 0};
    uint64_t steps = 0, packets = 0;
    uint32_t packet_steps = 0, iter = 0;
    uint32_t status = 0;

    uint64_t p = t;
    f3 pos, dir;
    float w, opl = 0.0f;
    int layer;
    uint32_t trace_count = 0, events = MCGB_EV_LAUNCH;
    mcml_launch(c, L, rng, pos, dir, w, layer, accu);
    if (use_trace && (c.trace.flags & MCGB_TRACE_START))
        trace_event(c.trace, p, trace_count, events, pos, dir, w, opl, b.float_buffer);

    for (;;) {
        const float4 g0 = L[layer].g0;   /* top, bottom, inv_mut, mua_inv_mut */
        ++packet_steps;
        ++iter;
        float u = rng.next();
        float step;
        if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT)
            step = mc_div(-mc_log(u), L[layer].g1.z);
        else
            step = -mc_log(u) * g0.z;
        step = fminf(step, FLT_MAX);
        int next = layer;
        if (pos.z + step * dir.z < g0.x) {
            --next;
            if (fabsf(dir.z) != 0.0f) step = mc_div(g0.x - pos.z, dir.z);
        }
        if (pos.z + step * dir.z >= g0.y) {
            ++next;
            if (fabsf(dir.z) != 0.0f) step = mc_div(g0.y - pos.z, dir.z);
        }
        pos.x = pos.x + dir.x * step;
        pos.y = pos.y + dir.y * step;
        pos.z = pos.z + dir.z * step;
        if (track_opl) opl += L[layer].g1.x * step;
        if (layer < next) pos.z = g0.y;
        if (layer > next) pos.z = g0.x;

        bool done = false;
        if (METHOD == MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT) {
            /* mcml.template.c:584-666 */
            float mua = L[layer].g1.y;
            float fraction = 1.0f - mc_exp(-mua * step);
            float deposit = fraction * w;
            w -= deposit;
            events |= MCGB_EV_ABSORPTION;
            if (FLU) {
                float step_back = (mua != 0.0f)
                                      ? step - mc_div(-mc_log(1.0f - rng.next() * fraction), mua)
                                      : 0.0f;
                f3 dp{pos.x - step_back * dir.x, pos.y - step_back * dir.y, pos.z - step_back * dir.z};
                fluence_deposit(c.fluence, dp, deposit, mua, accu, fcache);
            }
            if (next != layer) {
                events |= mcml_boundary(L, layer, next, dir, rng) | MCGB_EV_BOUNDARY_HIT;
                if (!(layer > 0 && layer < last_layer)) {
                    if (layer <= 0) detector_deposit(c.top, pos, dir, w, accu);
                    else detector_deposit(c.bottom, pos, dir, w, accu);
                    done = true;
                }
            } else {
                const MlLayer &cl = L[layer];
                float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, lut, rng, &az);
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
        } else if (next != layer) {
            events |= mcml_boundary(L, layer, next, dir, rng) | MCGB_EV_BOUNDARY_HIT;
            if (!(layer > 0 && layer < last_layer)) {
                if (layer <= 0) detector_deposit(c.top, pos, dir, w, accu);
                else detector_deposit(c.bottom, pos, dir, w, accu);
                done = true;
            }
        } else if (METHOD == MCGB_METHOD_ALBEDO_REJECTION) {
            /* mcml.template.c:705-721 */
            if (rng.next() < g0.w) {
                float deposit = w;
                done = true;
                w -= deposit;
                events |= MCGB_EV_ABSORPTION;
                if (FLU) fluence_deposit(c.fluence, pos, deposit, L[layer].g1.y, accu, fcache);
            } else {
                const MlLayer &cl = L[layer];
                float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, lut, rng, &az);
                scatter_direction(dir, ct, az);
                events |= MCGB_EV_SCATTERING;
            }
        } else {
            /* albedo weight, mcml.template.c:722-753 */
            float deposit = w * g0.w;
            w -= deposit;
            events |= MCGB_EV_ABSORPTION;
            if (FLU) fluence_deposit(c.fluence, pos, deposit, L[layer].g1.y, accu, fcache);
            const MlLayer &cl = L[layer];
            float az, ct = pf_sample<PF>(cl.pf0, cl.pf1, lut, rng, &az);
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
        /* rmax, mcml.template.c:759-763 */
        if (use_rmax) {
            f3 d{pos.x - src_pos.x, pos.y - src_pos.y, pos.z - src_pos.z};
            if (dot3(d, d) > rmax2) {
                done = true;
                events |= MCGB_EV_ESCAPED;
            }
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
            mcml_launch(c, L, rng, pos, dir, w, layer, accu);
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
