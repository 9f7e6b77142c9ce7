/* batch_launch.h - scratch layout and launchers of the batched engine. */
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include "../../include/xopto_gb300.h"

/* Scratch layout: [queue counter, 16 B][prefix sums, (S+1) x 8 B, padded to
   16 B][per-simulation tables, S x 256 B]. */
#define MCGB_BATCH_PREP_BYTES 256u

struct BatchWork {
    unsigned long long *queue;
    uint64_t *prefix;
    void *prep;
};

static inline uint64_t batch_work_bytes(uint32_t S) {
    uint64_t prefix = ((uint64_t)(S + 1) * 8u + 15u) / 16u * 16u;
    return 16u + prefix + (uint64_t)S * MCGB_BATCH_PREP_BYTES;
}

static inline BatchWork batch_work_layout(void *work, uint32_t S) {
    char *p = static_cast<char *>(work);
    BatchWork w;
    w.queue = reinterpret_cast<unsigned long long *>(p);
    w.prefix = reinterpret_cast<uint64_t *>(p + 16);
    w.prep = p + 16 + ((uint64_t)(S + 1) * 8u + 15u) / 16u * 16u;
    return w;
}

#define MCGB_DECLARE_BATCH(NS)                                                                 \
    namespace NS {                                                                           \
    cudaError_t launch_batched(const McgbBatchConfig &, const McgbBatchSim *, const uint32_t *, \
                               uint64_t *, void *, uint64_t *, cudaStream_t, unsigned, unsigned,\
                               uint64_t);                                                    \
    cudaError_t batched_occupancy(int block, int *blocks_per_sm);                            \
    size_t prep_record_bytes();                                                              \
    }
MCGB_DECLARE_BATCH(mcgb_exact_batch)
MCGB_DECLARE_BATCH(mcgb_fast_batch)
