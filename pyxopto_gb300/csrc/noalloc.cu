/*
 * noalloc.cu - a batched-engine entry point for callers that cannot
 * allocate device memory.
 *
 * mcgb_batched_run needs a scratch ("work") buffer besides its inputs and
 * outputs: the work-queue counter, the packet prefix sums and the
 * per-simulation layer tables.  Some callers cannot provide one: code that
 * runs inside another framework's memory pool or under a real-time loop
 * where cudaMalloc is forbidden (it can synchronize the device and can
 * stall or fail when the memory is reserved by another allocator), and plugin
 * hosts that hand over only input and output pointers.  For them,
 * mcgb_batched_run_noalloc keeps the scratch in a fixed device array inside
 * this library, sized for MCGB_NOALLOC_MAX_SIMS simulations (about 2.2 MB;
 * every GPU that loads the library holds it until the process exits).
 *
 * Host code cannot use the array's name as a device address, so the first
 * call on each device looks the address up with cudaGetSymbolAddress (with
 * that device current) and caches it together with the identity of the
 * device's current context; make that first call before any stream capture.
 * A device reset (cudaDeviceReset, or a release and re-creation of the
 * primary context) reloads the library's module at a new address, so the
 * next call sees a new context identity and looks the address up again; that
 * call, too, belongs before any stream capture.  All calls share the one array, so calls that overlap on
 * the GPU (different streams, or different host threads on the same device)
 * race on it and must be serialized by the caller.  The array keeps the last
 * call's contents; everything the kernels need zeroed (the work-queue
 * counter) is cleared by the preparation kernel of each call.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <mutex>
#include "../../include/xopto_gb300.h"
#include "batch_launch.h"
#include "errors.h"

namespace {

constexpr uint64_t kScratchBytes =
    16u + ((uint64_t)(MCGB_NOALLOC_MAX_SIMS + 1) * 8u + 15u) / 16u * 16u +
    (uint64_t)MCGB_NOALLOC_MAX_SIMS * MCGB_BATCH_PREP_BYTES;

constexpr int kMaxDevices = 64;

std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices];
unsigned long long g_scratch_ctx[kMaxDevices];   /* context identity of the cached address */

/* Identity of the calling thread's current context (cuCtxGetCurrent +
   cuCtxGetId, fetched through the runtime so that the library does not link
   libcuda).  Returns false when it cannot be told; the caller then
   looks the address up on every call. */
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

bool current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        resolved = true;
        void *f = nullptr, *g = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q1) ==
                cudaSuccess && q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) ==
                cudaSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
            get_id = reinterpret_cast<CtxGetIdFn>(g);
        }
    }
    if (!get_current || !get_id) return false;
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

}  // namespace

static __device__ __align__(256) unsigned char g_batch_scratch[kScratchBytes];

namespace {

/* Device address of g_batch_scratch on the current device: looked up once
   per device and context, again after a device reset. */
int scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mcgb_internal::set_error(MCGB_E_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices)
        return mcgb_internal::set_error(MCGB_E_UNSUPPORTED, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_mu);
    unsigned long long ctx = 0;
    bool known = current_context_id(&ctx);
    if (!g_scratch_ptr[dev] || !known || g_scratch_ctx[dev] != ctx) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_batch_scratch);
        if (e != cudaSuccess || !p)
            return mcgb_internal::set_error(MCGB_E_CUDA,
                                            "cudaGetSymbolAddress of the batched scratch array failed");
        /* the lookup may have created the context: take its identity now */
        known = current_context_id(&ctx);
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = known ? ctx : 0ull;
        if (!known) {
            *out = p;
            g_scratch_ptr[dev] = nullptr;
            return MCGB_OK;
        }
    }
    *out = g_scratch_ptr[dev];
    return MCGB_OK;
}

}  // namespace

extern "C" int mcgb_batched_run_noalloc(const McgbBatchConfig *cfg, const McgbBatchSim *dev_sims,
                                        const uint32_t *dev_multipliers, uint64_t *dev_tally,
                                        uint64_t *dev_counters, void *stream) {
    if (!cfg) return mcgb_internal::set_error(MCGB_E_INVALID, "cfg is NULL");
    if (cfg->num_sims > MCGB_NOALLOC_MAX_SIMS || batch_work_bytes(cfg->num_sims) > kScratchBytes)
        return mcgb_internal::set_error(
            MCGB_E_SIZE, "mcgb_batched_run_noalloc takes at most MCGB_NOALLOC_MAX_SIMS (8192) "
                         "simulations; use mcgb_batched_run with a caller-owned work buffer");
    void *work = nullptr;
    int r = scratch_address(&work);
    if (r) return r;
    return mcgb_batched_run(cfg, dev_sims, dev_multipliers, dev_tally, work, dev_counters, stream);
}
