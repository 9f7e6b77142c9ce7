/*
 * transport_exact.cu - layered and voxelized transport kernels compiled in
 * EXACT math: IEEE arithmetic without FMA contraction (built with -fmad=false)
 * and the portable log/exp/sincos/powr routines; bit-identical to a CPU
 * evaluation of the same algorithm.
 */
#define MCGB_FAST_MATH 0
#define MCGB_NS mcgb_exact
#include <cuda_runtime.h>
#include "mcml_kernel.cuh"
#include "mcvox_kernel.cuh"
#include "launch.h"

namespace mcgb_exact {

/* Kernel variants: scheduling x phase function x method x fluence. */
#define MCGB_V(K, PF, M) {(const void *)K<PF, M, false>, (const void *)K<PF, M, true>}
#define MCGB_METHODS(K, PF) {MCGB_V(K, PF, 0), MCGB_V(K, PF, 1), MCGB_V(K, PF, 2)}
#define MCGB_TABLE(K) {MCGB_METHODS(K, 0), MCGB_METHODS(K, 1), MCGB_METHODS(K, 2)}

static const void *const kMcml[2][3][3][2] = {MCGB_TABLE(mcml_transport_kernel),
                                              MCGB_TABLE(mcml_dynamic_kernel)};
static const void *const kMcvox[2][3][3][2] = {MCGB_TABLE(mcvox_transport_kernel),
                                               MCGB_TABLE(mcvox_dynamic_kernel)};

static const void *select(int medium, int sched, int pf, int method, bool fluence) {
    if (pf < 0 || pf > 2 || method < 0 || method > 2 || sched < 0 || sched > 1) return nullptr;
    return medium == 0 ? kMcml[sched][pf][method][fluence ? 1 : 0]
                       : kMcvox[sched][pf][method][fluence ? 1 : 0];
}

template <class Cfg>
static cudaError_t launch(int medium, const Cfg &cfg, const McgbBuffers &buf, cudaStream_t stream,
                          const LaunchShape &shape) {
    const int sched = cfg.opt.scheduling;
    const void *k = select(medium, sched, cfg.pf_kind, cfg.opt.method,
                           cfg.fluence.kind != MCGB_FLUENCE_NONE);
    if (!k) return cudaErrorInvalidValue;
    if (shape.dyn_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)shape.dyn_smem);
        if (e != cudaSuccess) return e;
    }
    unsigned grid = shape.grid;
    if (sched == MCGB_SCHED_DYNAMIC) {
        /* persistent: as many blocks as stay resident */
        int dev = 0, sms = 0, bps = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, (int)shape.block, shape.dyn_smem);
        if (e != cudaSuccess) return e;
        if (bps < 1) return cudaErrorInvalidConfiguration;
        grid = (unsigned)(sms * bps);
    }
    McgbBuffers b = buf;
    uint64_t deadline = shape.deadline_ns;
    int lut = shape.lut_in_smem;
    void *args[] = {(void *)&cfg, (void *)&b, (void *)&deadline, (void *)&lut};
    return cudaLaunchKernel(k, dim3(grid), dim3(shape.block), args, shape.dyn_smem, stream);
}

cudaError_t launch_mcml(const McgbMcmlConfig &cfg, const McgbBuffers &buf, cudaStream_t stream,
                        const LaunchShape &shape) {
    return launch(0, cfg, buf, stream, shape);
}

cudaError_t launch_mcvox(const McgbMcvoxConfig &cfg, const McgbBuffers &buf, cudaStream_t stream,
                         const LaunchShape &shape) {
    return launch(1, cfg, buf, stream, shape);
}

cudaError_t occupancy(int medium, int block, size_t dyn_smem, int *blocks_per_sm) {
    /* the smallest residency over the static variants of the medium, so that
       one wave of the suggested stream count fits whichever variant runs */
    int best = 1 << 30;
    for (int pf = 0; pf < 3; ++pf)
        for (int m = 0; m < 3; ++m)
            for (int fl = 0; fl < 2; ++fl) {
                int n = 0;
                cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &n, select(medium, MCGB_SCHED_STATIC, pf, m, fl != 0), block, dyn_smem);
                if (e != cudaSuccess) return e;
                best = n < best ? n : best;
            }
    *blocks_per_sm = best;
    return cudaSuccess;
}

}  // namespace mcgb_exact
