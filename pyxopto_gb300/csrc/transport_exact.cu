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

cudaError_t launch_mcml(const McgbMcmlConfig &cfg, const McgbBuffers &buf, cudaStream_t stream,
                        const LaunchShape &shape) {
    if (shape.dyn_smem > 48 * 1024)
        cudaFuncSetAttribute(mcml_transport_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)shape.dyn_smem);
    mcml_transport_kernel<<<shape.grid, shape.block, shape.dyn_smem, stream>>>(
        cfg, buf, shape.deadline_ns, shape.lut_in_smem);
    return cudaGetLastError();
}

cudaError_t launch_mcvox(const McgbMcvoxConfig &cfg, const McgbBuffers &buf, cudaStream_t stream,
                         const LaunchShape &shape) {
    if (shape.dyn_smem > 48 * 1024)
        cudaFuncSetAttribute(mcvox_transport_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)shape.dyn_smem);
    mcvox_transport_kernel<<<shape.grid, shape.block, shape.dyn_smem, stream>>>(
        cfg, buf, shape.deadline_ns, shape.lut_in_smem);
    return cudaGetLastError();
}

cudaError_t occupancy(int medium, int block, size_t dyn_smem, int *blocks_per_sm) {
    if (medium == 0)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mcml_transport_kernel,
                                                             block, dyn_smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mcvox_transport_kernel,
                                                         block, dyn_smem);
}

}  // namespace mcgb_exact
