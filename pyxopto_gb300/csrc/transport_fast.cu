/*
 * transport_fast.cu - layered and voxelized transport kernels compiled in
 * FAST math: special-function-unit log2/sin/cos/ex2 and approximate division
 * and square root (built with -use_fast_math); the reference's
 * MC_USE_NATIVE_MATH.
 */
#define MCGB_FAST_MATH 1
#define MCGB_NS mcgb_fast
#include <cuda_runtime.h>
#include "mcml_kernel.cuh"
#include "mcvox_kernel.cuh"
#include "launch.h"

namespace mcgb_fast {

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

}  // namespace mcgb_fast
