// Sampling volume of packet traces: the reference's SamplingVolume kernel
// (xopto/mcbase/kernel/mcsv.template.c:236-421) re-planned for GB300.
//
// One thread walks one packet's recorded path voxel by voxel, exactly in the
// reference's order (the voxel index is carried from event to event and the
// length inside a voxel is summed across events), so the integer tallies are
// identical to the CPU restatement.  Parallelism is across packets: a walk
// cannot be split by segment without changing the float sums.
//
// Layout: the trace is packet-major, max_events events of 8 floats per packet
// (32 B per event, read as two float4 with streaming loads so the one-pass
// trace does not evict the voxel tallies from L2).  The tallies are 64-bit
// integers updated with atomics; a 200^3 volume is 64 MB and stays in L2.
//
// Compiled without contraction (-fmad=false) and with IEEE division and
// square root: the walk compares distances, and a fused multiply-add would
// move a crossing to another voxel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xopto_gb300.h"

namespace {

constexpr uint32_t kMaxCrossings = MCGB_SV_MAX_CROSSINGS;

struct SvEvent {
    float px, py, pz, dx, dy, dz;
};

__device__ __forceinline__ void sv_load(const float *packet, int32_t i, SvEvent &e) {
    const float4 *p = reinterpret_cast<const float4 *>(packet + (size_t)i * MCGB_TRACE_ENTRY_LEN);
    float4 a = __ldcs(p);
    float4 b = __ldcs(p + 1);
    e.px = a.x; e.py = a.y; e.pz = a.z;
    e.dx = a.w; e.dy = b.x; e.dz = b.y;
}

// mc_distance_fpv3 (xopto/mcbase/kernel/mcbase.template.c:1061-1064).
__device__ __forceinline__ float sv_distance(const SvEvent &a, const SvEvent &b) {
    float x = a.px - b.px, y = a.py - b.py, z = a.pz - b.pz;
    return sqrtf(x * x + y * y + z * z);
}

// Float to integer conversions truncate toward zero and saturate (a negative
// weight becomes 0), the device behaviour of the reference's casts.
__device__ __forceinline__ uint32_t sv_weight(float w) { return __float2uint_rz(w); }

struct SvVoxel {
    int32_t x, y, z;
};

// sva_intersect (mcsv.template.c:97-120): distance along the direction to the
// exit wall of the current voxel on each axis.
__device__ __forceinline__ float sv_wall(float top_left, int32_t v, float size, float pos,
                                         float dir) {
    float d = top_left + (float)((int32_t)(dir >= 0.0f) + v) * size - pos;
    return dir != 0.0f ? d / dir : __int_as_float(0x7f800000);
}

__global__ void __launch_bounds__(128)
sampling_volume_kernel(McgbSamplingVolume sv, const float *__restrict__ trace,
                       const int32_t *__restrict__ counts, uint64_t *__restrict__ accu,
                       uint64_t *__restrict__ total_weight, uint64_t *__restrict__ counters) {
    const float k = (float)sv.k;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < sv.num_packets;
         p += stride) {
        int32_t n = counts[p];
        if (n > (int32_t)sv.max_events) n = (int32_t)sv.max_events;
        if (n <= 0) continue;
        const float *tr = trace + p * (uint64_t)sv.max_events * MCGB_TRACE_ENTRY_LEN;
        // "end weight": the last float of the last event (mcsv.template.c:299)
        const float end_w = __ldcs(tr + (size_t)n * MCGB_TRACE_ENTRY_LEN - 1);
        atomicAdd((unsigned long long *)total_weight,
                  (unsigned long long)sv_weight(end_w * k + 0.5f));

        SvEvent e1, e2;
        int32_t ei = 0;
        sv_load(tr, 0, e1);
        sv_load(tr, n > 1 ? 1 : n - 1, e2);
        float d12 = sv_distance(e1, e2);
        SvVoxel v;
        v.x = __float2int_rz((e1.px - sv.top_left[0]) / sv.voxel_size[0]);
        v.y = __float2int_rz((e1.py - sv.top_left[1]) / sv.voxel_size[1]);
        v.z = __float2int_rz((e1.pz - sv.top_left[2]) / sv.voxel_size[2]);
        float l_voxel = 0.0f;
        uint32_t crossings = 0;

        while (true) {
            float dx = sv_wall(sv.top_left[0], v.x, sv.voxel_size[0], e1.px, e1.dx);
            float dy = sv_wall(sv.top_left[1], v.y, sv.voxel_size[1], e1.py, e1.dy);
            float dz = sv_wall(sv.top_left[2], v.z, sv.voxel_size[2], e1.pz, e1.dz);
            float d_voxel = fminf(dz, fminf(dx, dy));
            float d_move = fminf(d_voxel, d12);
            l_voxel += d_move;
            bool leaving = d_voxel < d12;
            bool last = false;
            if (!leaving) {
                e1 = e2;
                ++ei;
                if (ei < n - 1) {
                    sv_load(tr, ei + 1, e2);
                    d12 = sv_distance(e1, e2);
                    continue;
                }
                last = true;
            }
            // leaving the voxel, or the path ended inside it: deposit
            // (sva_deposit_weight, mcsv.template.c:198-202)
            if (v.x >= 0 && v.y >= 0 && v.z >= 0 && (uint32_t)v.x < sv.shape[0] &&
                (uint32_t)v.y < sv.shape[1] && (uint32_t)v.z < sv.shape[2]) {
                uint64_t index = ((uint64_t)v.z * sv.shape[1] + (uint64_t)v.y) * sv.shape[0] +
                                 (uint64_t)v.x;
                uint32_t w = sv_weight(end_w * l_voxel * sv.multiplier * k + 0.5f);
                if (w) atomicAdd((unsigned long long *)(accu + sv.offset + index),
                                 (unsigned long long)w);
            }
            if (last) break;
            e1.px += e1.dx * d_move;
            e1.py += e1.dy * d_move;
            e1.pz += e1.dz * d_move;
            d12 -= d_move;
            // sva_next_voxel (mcsv.template.c:136-160): step across the
            // nearest wall; ties go to x, then y.
            int32_t nx = (dx <= dy) && (dx <= dz);
            int32_t ny = nx ? 0 : ((dy <= dx) && (dy <= dz));
            int32_t nz = !(nx + ny);
            v.x += e1.dx < 0.0f ? -nx : nx;
            v.y += e1.dy < 0.0f ? -ny : ny;
            v.z += e1.dz < 0.0f ? -nz : nz;
            l_voxel = 0.0f;
            if (++crossings >= kMaxCrossings) {
                if (counters)
                    atomicOr((unsigned long long *)(counters + MCGB_CNT_STATUS),
                             (unsigned long long)MCGB_STATUS_BAD_INDEX);
                break;
            }
        }
    }
}

}  // namespace

namespace mcgb_sv {

cudaError_t launch(const McgbSamplingVolume &sv, const float *trace, const int32_t *counts,
                   uint64_t *accu, uint64_t *total_weight, uint64_t *counters,
                   cudaStream_t stream) {
    if (sv.num_packets == 0) return cudaSuccess;
    int device = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    uint64_t blocks = (sv.num_packets + 127) / 128;
    uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 16;
    if (blocks > cap) blocks = cap;
    sampling_volume_kernel<<<(unsigned)blocks, 128, 0, stream>>>(sv, trace, counts, accu,
                                                                total_weight, counters);
    return cudaGetLastError();
}

}  // namespace mcgb_sv
