/* launch.h - launch shape passed from the C ABI layer to the kernel
 * translation units (one per medium and math mode). */
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include "../../include/xopto_gb300.h"

struct LaunchShape {
    unsigned grid;
    unsigned block;
    size_t dyn_smem;
    int lut_in_smem;
    uint64_t deadline_ns;   /* run time limit measured from each thread's start */
};

#define MCGB_DECLARE_LAUNCHERS(NS)                                                             \
    namespace NS {                                                                           \
    cudaError_t launch_mcml(const McgbMcmlConfig &, const McgbBuffers &, cudaStream_t,       \
                            const LaunchShape &);                                            \
    cudaError_t launch_mcvox(const McgbMcvoxConfig &, const McgbBuffers &, cudaStream_t,     \
                             const LaunchShape &);                                           \
    cudaError_t occupancy_mcml(int block, size_t dyn_smem, int *blocks_per_sm);              \
    cudaError_t occupancy_mcvox(int block, size_t dyn_smem, int *blocks_per_sm);             \
    }
MCGB_DECLARE_LAUNCHERS(mcgb_exact)
MCGB_DECLARE_LAUNCHERS(mcgb_fast)
