/*
 * batched.cu - the batched engine compiled in FAST math (-use_fast_math).
 */
#define MCGB_FAST_MATH 1
#define MCGB_NS mcgb_fast_batch
#include <cuda_runtime.h>
#include <cmath>
#include "batched_kernel.cuh"
#include "batch_launch.h"

namespace mcgb_fast_batch {

cudaError_t launch_batched(const McgbBatchConfig &cfg, const McgbBatchSim *sims, const uint32_t *mult,
                           uint64_t *tally, void *work, uint64_t *counters, cudaStream_t stream,
                           unsigned grid, unsigned block, uint64_t deadline_ns) {
    BatchWork wk = batch_work_layout(work, cfg.num_sims);
    batch_prep_kernel<<<1, 1024, 0, stream>>>(sims, cfg.num_sims, wk.prefix,
                                              reinterpret_cast<BatchPrep *>(wk.prep), wk.queue);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bool rmax = !std::isinf(cfg.rmax);
    if (rmax)
        batched_kernel<true><<<grid, block, 0, stream>>>(cfg, mult, wk.prefix,
            reinterpret_cast<const BatchPrep *>(wk.prep), wk.queue, tally, counters, deadline_ns);
    else
        batched_kernel<false><<<grid, block, 0, stream>>>(cfg, mult, wk.prefix,
            reinterpret_cast<const BatchPrep *>(wk.prep), wk.queue, tally, counters, deadline_ns);
    return cudaGetLastError();
}

cudaError_t batched_occupancy(int block, int *blocks_per_sm) {
    int a = 0, b = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, batched_kernel<true>, block, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_kernel<false>, block, 0);
    *blocks_per_sm = a < b ? a : b;
    return e;
}

size_t prep_record_bytes() { return sizeof(BatchPrep); }

}  // namespace mcgb_fast_batch
