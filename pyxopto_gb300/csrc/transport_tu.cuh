/*
 * transport_tu.cuh - kernel tables and launcher of one medium in one math
 * mode.  Included by the eight translation units
 * transport_{exact,fast}_{mcml,mcvox}_{static,dynamic}.cu, which define
 * MCGB_FAST_MATH, MCGB_NS, MCGB_MEDIUM (0 layered, 1 voxelized) and
 * MCGB_PART (0 the static-scheduling kernels, 1 the dynamic-scheduling
 * kernels and the launcher), so that the kernel variants compile in parallel.
 */
#pragma once
#include <cuda_runtime.h>
#include <limits>
#include <mutex>
#include "launch.h"
#if MCGB_MEDIUM == 0
#include "mcml_kernel.cuh"
#define MCGB_STATIC_KERNEL mcml_transport_kernel
#define MCGB_DYNAMIC_KERNEL mcml_dynamic_kernel
#define MCGB_CFG McgbMcmlConfig
#define MCGB_LAUNCH launch_mcml
#define MCGB_OCCUPANCY occupancy_mcml
#define MCGB_SELECT_STATIC select_static_mcml
#else
#include "mcvox_kernel.cuh"
#define MCGB_STATIC_KERNEL mcvox_transport_kernel
#define MCGB_DYNAMIC_KERNEL mcvox_dynamic_kernel
#define MCGB_CFG McgbMcvoxConfig
#define MCGB_LAUNCH launch_mcvox
#define MCGB_OCCUPANCY occupancy_mcvox
#define MCGB_SELECT_STATIC select_static_mcvox
#endif

namespace MCGB_NS {

#define MCGB_METHODS(V, K, PF) {V(K, PF, 0), V(K, PF, 1), V(K, PF, 2)}
#define MCGB_TABLE(V, K) {MCGB_METHODS(V, K, 0), MCGB_METHODS(V, K, 1), MCGB_METHODS(V, K, 2), \
                          MCGB_METHODS(V, K, 3)}

/* Static scheduling kernels: phase function x method x fluence; they carry
   every optional feature and every source. */
const void *MCGB_SELECT_STATIC(int pf, int method, bool fluence);

#if MCGB_PART == 0

#define MCGB_VS(K, PF, M) {(const void *)K<PF, M, false>, (const void *)K<PF, M, true>}
static const void *const kStatic[4][3][2] = MCGB_TABLE(MCGB_VS, MCGB_STATIC_KERNEL);

const void *MCGB_SELECT_STATIC(int pf, int method, bool fluence) {
    if (pf < 0 || pf > 3 || method < 0 || method > 2) return nullptr;
    return kStatic[pf][method][fluence ? 1 : 0];
}

#else

/* Dynamic scheduling kernels: phase function x method x fluence x optional
   features (trace, optical path length, per-packet step limit, fibre-probe
   detectors, surface layouts, fluence rate) x simple launch (the common
   sources only: Line in layered media, Line and GaussianBeam in voxelized
   media; no rmax). */
#define MCGB_VX(K, PF, M, F) {{(const void *)K<PF, M, F, false, false>, (const void *)K<PF, M, F, false, true>}, \
                              {(const void *)K<PF, M, F, true, false>, (const void *)K<PF, M, F, true, true>}}
#define MCGB_VD(K, PF, M) {MCGB_VX(K, PF, M, false), MCGB_VX(K, PF, M, true)}
static const void *const kDynamic[4][3][2][2][2] = MCGB_TABLE(MCGB_VD, MCGB_DYNAMIC_KERNEL);

static const void *select(int sched, int pf, int method, bool fluence, bool xtra, bool simple) {
    if (pf < 0 || pf > 3 || method < 0 || method > 2 || sched < 0 || sched > 1) return nullptr;
    if (sched == MCGB_SCHED_STATIC) return MCGB_SELECT_STATIC(pf, method, fluence);
    return kDynamic[pf][method][fluence ? 1 : 0][xtra ? 1 : 0][simple ? 1 : 0];
}

static bool simple_source(int kind) {
#if MCGB_MEDIUM == 0
    return kind == MCGB_SRC_LINE;
#else
    return kind == MCGB_SRC_LINE || kind == MCGB_SRC_GAUSSIAN_BEAM;
#endif
}

/* Resident blocks per SM of a kernel variant for a block size, queried once
   per (device, variant, block size) and remembered. */
static cudaError_t resident_blocks(const void *k, int block, size_t dyn_smem, int *bps) {
    struct Entry { int dev; const void *k; int block; size_t smem; int bps; };
    static std::mutex lock;
    static Entry cache[64];
    static int used = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> g(lock);
        for (int i = 0; i < used; ++i)
            if (cache[i].dev == dev && cache[i].k == k && cache[i].block == block &&
                cache[i].smem == dyn_smem) {
                *bps = cache[i].bps;
                return cudaSuccess;
            }
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, block, dyn_smem);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(lock);
    if (used < 64) cache[used++] = Entry{dev, k, block, dyn_smem, *bps};
    return cudaSuccess;
}

cudaError_t MCGB_LAUNCH(const MCGB_CFG &cfg, const McgbBuffers &buf, cudaStream_t stream,
                        const LaunchShape &shape) {
    const int sched = cfg.opt.scheduling;
    /* the plain dynamic kernels (XTRA = false) also leave out the
       fluence-rate scaling, and the SIMPLE ones the rmax test */
    const float rmax2 = cfg.opt.rmax * cfg.opt.rmax;
    const bool rmax = rmax2 < std::numeric_limits<float>::infinity();
    bool xtra = cfg.trace.flags != MCGB_TRACE_NONE || cfg.opt.track_optical_pathlength != 0 ||
                cfg.opt.max_steps_per_packet != 0 || cfg.fluence.kind == MCGB_FLUENCE_RATE;
    xtra = xtra || cfg.top.kind >= MCGB_DET_LINEAR_ARRAY || cfg.bottom.kind >= MCGB_DET_LINEAR_ARRAY;
#if MCGB_MEDIUM == 0
    xtra = xtra || cfg.surface_top.kind != MCGB_SURFACE_NONE ||
           cfg.surface_bottom.kind != MCGB_SURFACE_NONE;
#endif
    const void *k = select(sched, cfg.pf_kind, cfg.opt.method, cfg.fluence.kind != MCGB_FLUENCE_NONE,
                           xtra, simple_source(cfg.source.kind) && !rmax);
    if (!k) return cudaErrorInvalidValue;
    if (shape.dyn_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)shape.dyn_smem);
        if (e != cudaSuccess) return e;
    }
    unsigned grid = shape.grid, block = shape.block;
    if (sched == MCGB_SCHED_DYNAMIC) {
        /* persistent: as many 128-thread blocks as stay resident (the
           dynamic kernels are compiled for 128-thread blocks) */
        block = 128;
        int dev = 0, sms = 0, bps = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = resident_blocks(k, (int)block, shape.dyn_smem, &bps);
        if (e != cudaSuccess) return e;
        if (bps < 1) return cudaErrorInvalidConfiguration;
        grid = (unsigned)(sms * bps);
    }
    /* dynamic scheduling: packets per queue item; by default at least 4
       items per warp of the grid (so that short runs still spread over every
       warp), at most 128 (one queue access per 128 packets in long runs) */
    uint32_t items = cfg.opt.packets_per_item;
    if (items == 0) {
        uint64_t warps = (uint64_t)grid * (block / 32u);
        uint64_t b = cfg.num_packets / (warps * 4u);
        items = (uint32_t)(b < 1 ? 1 : (b > 128 ? 128 : b));
    }
    McgbBuffers b = buf;
    uint64_t deadline = shape.deadline_ns;
    int lut = shape.lut_in_smem;
    void *args[] = {(void *)&cfg, (void *)&b, (void *)&deadline, (void *)&lut, (void *)&items};
    return cudaLaunchKernel(k, dim3(grid), dim3(block), args, shape.dyn_smem, stream);
}

cudaError_t MCGB_OCCUPANCY(int block, size_t dyn_smem, int *blocks_per_sm) {
    /* the smallest residency over the static variants of the medium, so that
       one wave of the suggested stream count fits whichever variant runs */
    int best = 1 << 30;
    for (int pf = 0; pf <= MCGB_PF_EXT; ++pf)
        for (int m = 0; m < 3; ++m)
            for (int fl = 0; fl < 2; ++fl) {
                int n = 0;
                cudaError_t e = resident_blocks(MCGB_SELECT_STATIC(pf, m, fl != 0), block, dyn_smem, &n);
                if (e != cudaSuccess) return e;
                best = n < best ? n : best;
            }
    *blocks_per_sm = best;
    return cudaSuccess;
}

#endif

}  // namespace MCGB_NS
