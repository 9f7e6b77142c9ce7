/*
 * capi.cu - the C ABI of libxopto_gb300.so (declared in
 * include/xopto_gb300.h): argument validation, launch shapes, status
 * checks, and the small utility kernels (random-number dump, buffer fill).
 *
 * Host-side checks mirror the reference's failure detection: struct-size
 * handshake (xopto/mcml/mc.py:674-728), packet-count limit (mc.py:813-818),
 * LUT/option consistency (mc.py:887-898).  Every offset a configuration names
 * is checked against the buffer sizes before a kernel is launched, so the
 * kernels index only memory the caller handed over.
 */
#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include "../../include/xopto_gb300.h"
#include "launch.h"
#include "errors.h"
#include "batch_launch.h"

namespace mcgb_sv {
cudaError_t launch(const McgbSamplingVolume &sv, const float *trace, const int32_t *counts,
                   uint64_t *accu, uint64_t *total_weight, uint64_t *counters, cudaStream_t stream);
}

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(MCGB_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

bool range_ok(uint64_t offset, uint64_t count, uint64_t size) {
    return offset <= size && count <= size - offset;
}

int check_pf(int kind, const McgbPf &pf, const McgbBuffers *b, const char *who, unsigned idx) {
    if (kind == MCGB_PF_EXT && pf.ext_kind > MCGB_PF_EXT_HGDIR)
        return fail(MCGB_E_INVALID, "%s %u: unknown analytic phase function %u", who, idx, pf.ext_kind);
    if (kind == MCGB_PF_EXT && (pf.ext_kind == MCGB_PF_EXT_GK2 || pf.ext_kind == MCGB_PF_EXT_HGA)) {
        uint32_t n = pf.ext_kind == MCGB_PF_EXT_GK2 ? MCGB_PF_GK2_FLOATS : MCGB_PF_HGA_FLOATS;
        if (!b->fp_lut || !range_ok(pf.lut_offset, n, b->fp_lut_size))
            return fail(MCGB_E_SIZE, "%s %u: phase-function parameters [%u, +%u) beyond the LUT buffer "
                        "(%llu floats)", who, idx, pf.lut_offset, n, (unsigned long long)b->fp_lut_size);
    }
    if (kind == MCGB_PF_LUT) {
        if (!b->fp_lut) return fail(MCGB_E_INVALID, "%s %u: Lut phase function without a LUT buffer", who, idx);
        if (pf.lut_size < 2) return fail(MCGB_E_INVALID, "%s %u: Lut size %u < 2", who, idx, pf.lut_size);
        if (!range_ok(pf.lut_offset, pf.lut_size, b->fp_lut_size))
            return fail(MCGB_E_SIZE, "%s %u: LUT [%u, +%u) beyond the LUT buffer (%llu floats)", who, idx,
                        pf.lut_offset, pf.lut_size, (unsigned long long)b->fp_lut_size);
    }
    return MCGB_OK;
}

/* Floats that a surface layout of kind/n_fibers needs in the float table. */
uint64_t surface_floats(int kind, uint32_t n_fibers) {
    switch (kind) {
        case MCGB_SURFACE_LAMBERTIAN: return 2;
        case MCGB_SURFACE_LINEAR_ARRAY: return 31;
        case MCGB_SURFACE_SIX_AROUND_ONE: return 23;
        case MCGB_SURFACE_FIBER_ARRAY: return 4 + (uint64_t)MCGB_SURFACE_FIBER_FLOATS * n_fibers;
        default: return 0;
    }
}

int check_surface(const McgbSurface &sf, const McgbBuffers *b, const char *where) {
    if (sf.kind == MCGB_SURFACE_NONE) return MCGB_OK;
    if (sf.kind < MCGB_SURFACE_LAMBERTIAN || sf.kind > MCGB_SURFACE_FIBER_ARRAY)
        return fail(MCGB_E_INVALID, "%s surface layout: unknown kind %d", where, sf.kind);
    if ((sf.kind == MCGB_SURFACE_LINEAR_ARRAY || sf.kind == MCGB_SURFACE_FIBER_ARRAY) &&
        (sf.n_fibers == 0 || sf.n_fibers > 4096))
        return fail(MCGB_E_INVALID, "%s surface layout: %u fibres outside [1, 4096]", where, sf.n_fibers);
    uint64_t need = surface_floats(sf.kind, sf.n_fibers);
    if (sf.table_size < need)
        return fail(MCGB_E_SIZE, "%s surface layout: table of %u floats, %llu needed", where, sf.table_size,
                    (unsigned long long)need);
    if (!b->fp_lut || !range_ok(sf.table_offset, sf.table_size, b->fp_lut_size))
        return fail(MCGB_E_SIZE, "%s surface layout: table [%u, +%u) beyond the float table (%llu)", where,
                    sf.table_offset, sf.table_size, (unsigned long long)b->fp_lut_size);
    return MCGB_OK;
}

int check_common(const McgbRunOptions &o, int pf_kind, uint64_t num_packets, uint32_t num_streams,
                 const McgbSource &src, const McgbDetector *dets, const McgbFluence &fl,
                 const McgbTrace &tr, const McgbBuffers *b) {
    if (!b) return fail(MCGB_E_INVALID, "buffers is NULL");
    if (num_streams == 0) return fail(MCGB_E_INVALID, "num_streams must be positive");
    if (num_streams > (1u << 24)) return fail(MCGB_E_SIZE, "num_streams %u exceeds 2^24", num_streams);
    if (o.scheduling != MCGB_SCHED_STATIC && o.scheduling != MCGB_SCHED_DYNAMIC)
        return fail(MCGB_E_INVALID, "unknown scheduling %d", o.scheduling);
    if (o.packets_per_item > 128)
        return fail(MCGB_E_INVALID, "packets per item %u outside [0, 128]", o.packets_per_item);
    if (!b->rng_a) return fail(MCGB_E_INVALID, "RNG multiplier buffer is NULL");
    if (o.scheduling == MCGB_SCHED_STATIC && !b->rng_x)
        return fail(MCGB_E_INVALID, "RNG state buffer is NULL");
    if (!b->counters) return fail(MCGB_E_INVALID, "counters buffer is NULL");
    if (o.method < 0 || o.method > 2) return fail(MCGB_E_INVALID, "unknown method %d", o.method);
    if (o.math != MCGB_MATH_EXACT && o.math != MCGB_MATH_FAST)
        return fail(MCGB_E_INVALID, "unknown math mode %d", o.math);
    if (pf_kind < 0 || pf_kind > MCGB_PF_EXT) return fail(MCGB_E_INVALID, "unknown phase function %d", pf_kind);
    if (src.kind < MCGB_SRC_LINE || src.kind > MCGB_SRC_ISOTROPIC_VOXELS)
        return fail(MCGB_E_INVALID, "unknown source kind %d", src.kind);
    if (src.kind >= MCGB_SRC_UNIFORM_FIBER_LUT_NI) {
        const uint64_t floats = (uint64_t)src.lut_size * (src.kind == MCGB_SRC_ISOTROPIC_VOXELS ? 4u : 1u);
        if (src.lut_size == 0 || src.lut_size > (1u << 24) || !b->fp_lut ||
            !range_ok(src.lut_offset, floats, b->fp_lut_size))
            return fail(MCGB_E_SIZE, "source table [%u, +%llu) beyond the float table (%llu)",
                        src.lut_offset, (unsigned long long)floats, (unsigned long long)b->fp_lut_size);
        if (src.kind != MCGB_SRC_UNIFORM_RECTANGULAR_LUT && src.kind != MCGB_SRC_ISOTROPIC_VOXELS &&
            !(src.sigma[0] >= 0.0f && src.clip > 0.0f))
            return fail(MCGB_E_INVALID, "fiber source: core radius %g, core index %g",
                        (double)src.sigma[0], (double)src.clip);
    }
    if (src.kind >= MCGB_SRC_UNIFORM_FIBER_NI && src.kind <= MCGB_SRC_LAMBERTIAN_FIBER &&
        !(src.sigma[0] >= 0.0f && src.sigma[1] >= 0.0f && src.sigma[1] <= 1.0f && src.clip > 0.0f))
        return fail(MCGB_E_INVALID, "fiber source: core radius %g, angular parameter %g, core index %g",
                    (double)src.sigma[0], (double)src.sigma[1], (double)src.clip);

    if (!(o.lottery_chance > 0.0f && o.lottery_chance <= 1.0f))
        return fail(MCGB_E_INVALID, "lottery chance %g outside (0, 1]", (double)o.lottery_chance);
    if (!(o.packet_weight_min > 0.0f && o.packet_weight_min <= 1.0f))
        return fail(MCGB_E_INVALID, "minimum packet weight %g outside (0, 1]", (double)o.packet_weight_min);
    if (num_packets > 0 && num_packets > UINT64_MAX - num_streams)
        return fail(MCGB_E_SIZE, "packet count overflows the packet index");
    const char *names[3] = {"top", "bottom", "specular"};
    for (int i = 0; i < 3; ++i) {
        const McgbDetector &d = dets[i];
        if (d.kind == MCGB_DET_NONE) continue;
        if (d.kind < MCGB_DET_TOTAL || d.kind > MCGB_DET_FIBER_LUT_ARRAY)
            return fail(MCGB_E_INVALID, "%s detector: unknown kind %d", names[i], d.kind);
        const bool pl = d.kind == MCGB_DET_RADIAL_PL || d.kind == MCGB_DET_TOTAL_PL ||
                        d.kind == MCGB_DET_CARTESIAN_PL || d.kind == MCGB_DET_LINEAR_ARRAY_PL ||
                        d.kind == MCGB_DET_SIX_AROUND_ONE_PL || d.kind == MCGB_DET_FIBER_ARRAY_PL ||
                        d.kind == MCGB_DET_TOTAL_LUT_PL;
        if (d.kind >= MCGB_DET_LINEAR_ARRAY && i == 2)
            return fail(MCGB_E_INVALID, "the specular slot takes no fibre-probe or look-up-table detector");
        if (d.kind >= MCGB_DET_TOTAL_LUT) {
            const bool fibers = d.kind == MCGB_DET_FIBER_LUT_ARRAY;
            if (fibers ? (d.n == 0 || d.n > 4096) : d.n != 1)
                return fail(MCGB_E_INVALID, "%s look-up-table detector: n = %u", names[i], d.n);
            if (d.n_y == 0 || (fibers && d.n_y < (uint64_t)MCGB_DET_LUT_FIBER_FLOATS * d.n))
                return fail(MCGB_E_INVALID, "%s look-up-table detector: table of %u floats", names[i], d.n_y);
            if (!b->fp_lut || !range_ok(d.table_offset, d.n_y, b->fp_lut_size))
                return fail(MCGB_E_SIZE, "%s look-up-table detector table [%u, +%u) beyond the float table",
                            names[i], d.table_offset, d.n_y);
        } else if (d.kind >= MCGB_DET_LINEAR_ARRAY) {
            const int base = d.kind >= MCGB_DET_LINEAR_ARRAY_PL ? d.kind - 3 : d.kind;
            if (base == MCGB_DET_SIX_AROUND_ONE && d.n != 7)
                return fail(MCGB_E_INVALID, "%s six-around-one detector needs n = 7", names[i]);
            if (d.n == 0 || d.n > 4096)
                return fail(MCGB_E_INVALID, "%s probe detector: %u fibres outside [1, 4096]", names[i], d.n);
            uint64_t floats = base == MCGB_DET_LINEAR_ARRAY     ? 15
                              : base == MCGB_DET_SIX_AROUND_ONE ? 14
                                                                : (uint64_t)MCGB_DET_FIBER_FLOATS * d.n;
            if (!b->fp_lut || !range_ok(d.table_offset, floats, b->fp_lut_size))
                return fail(MCGB_E_SIZE, "%s probe detector table [%u, +%llu) beyond the float table", names[i],
                            d.table_offset, (unsigned long long)floats);
        }
        if (pl) {
            if (!o.track_optical_pathlength)
                return fail(MCGB_E_INVALID, "%s path-length detector needs track_optical_pathlength",
                            names[i]);
            if (i == 2) return fail(MCGB_E_INVALID, "the specular slot takes no path-length detector");
        }
        uint64_t nr = 1;
        if (d.kind == MCGB_DET_RADIAL || d.kind == MCGB_DET_RADIAL_PL || d.kind == MCGB_DET_CARTESIAN ||
            d.kind == MCGB_DET_CARTESIAN_PL || d.kind >= MCGB_DET_LINEAR_ARRAY)
            nr = d.n;
        else if (d.kind == MCGB_DET_SYMMETRIC_X)
            nr = 2ull * d.n;
        uint64_t ny = (d.kind == MCGB_DET_CARTESIAN || d.kind == MCGB_DET_CARTESIAN_PL) ? d.n_y : 1;
        uint64_t npl = pl ? d.n_pl : 1;
        if (nr > 0x7FFFFFFFu || ny > 0x7FFFFFFFu || npl > 0x7FFFFFFFu || nr * ny * npl > 0xFFFFFFFFull)
            return fail(MCGB_E_SIZE, "%s detector has too many bins", names[i]);
        uint64_t n = nr * ny * npl;
        if (n == 0) return fail(MCGB_E_INVALID, "%s detector has no bins", names[i]);
        if (!b->accumulator || !range_ok(d.offset, n, b->accumulator_size))
            return fail(MCGB_E_SIZE, "%s detector [%llu, +%llu) beyond the accumulator (%llu)", names[i],
                        (unsigned long long)d.offset, (unsigned long long)n,
                        (unsigned long long)b->accumulator_size);
    }
    if (fl.kind != MCGB_FLUENCE_NONE) {
        if (fl.kind != MCGB_FLUENCE_DEPOSITION && fl.kind != MCGB_FLUENCE_RATE)
            return fail(MCGB_E_INVALID, "unknown fluence kind %d", fl.kind);
        if (fl.shape[0] == 0 || fl.shape[1] == 0 || fl.shape[2] == 0)
            return fail(MCGB_E_INVALID, "fluence grid has an empty axis");
        /* the kernels index the grid with 32-bit voxel numbers; 0xFFFFFFFF
           marks an empty fluence cache */
        uint64_t nxy = (uint64_t)fl.shape[0] * fl.shape[1];
        if (fl.shape[0] > 0x7FFFFFFFu || fl.shape[1] > 0x7FFFFFFFu || fl.shape[2] > 0x7FFFFFFFu ||
            nxy >= 0xFFFFFFFFull || nxy * fl.shape[2] >= 0xFFFFFFFFull)
            return fail(MCGB_E_SIZE, "fluence grid %ux%ux%u has 2^32 - 1 or more voxels", fl.shape[0],
                        fl.shape[1], fl.shape[2]);
        uint64_t n = nxy * fl.shape[2];
        if (!b->accumulator || !range_ok(fl.offset, n, b->accumulator_size))
            return fail(MCGB_E_SIZE, "fluence [%llu, +%llu) beyond the accumulator (%llu)",
                        (unsigned long long)fl.offset, (unsigned long long)n,
                        (unsigned long long)b->accumulator_size);
        if (fl.k <= 0) return fail(MCGB_E_INVALID, "fluence k must be positive");
    }
    if (tr.flags != MCGB_TRACE_NONE) {
        if (tr.max_events == 0) return fail(MCGB_E_INVALID, "trace max_events must be positive");
        if (num_packets > (UINT64_MAX / MCGB_TRACE_ENTRY_LEN) / tr.max_events)
            return fail(MCGB_E_SIZE, "trace size overflows");
        uint64_t nf = num_packets * tr.max_events * MCGB_TRACE_ENTRY_LEN;
        if (!b->float_buffer || !range_ok(tr.data_offset, nf, b->float_size))
            return fail(MCGB_E_SIZE, "trace events beyond the float buffer");
        if (!b->int_buffer || !range_ok(tr.count_offset, num_packets, b->int_size))
            return fail(MCGB_E_SIZE, "trace counts beyond the int buffer");
    }
    return MCGB_OK;
}

int device_sm_count(int *sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    return MCGB_OK;
}

int make_shape(int medium, int math, uint32_t block_size, uint32_t num_streams, const McgbBuffers *b,
               double deadline_s, LaunchShape *s) {
    s->block = block_size ? block_size : 128;
    if (s->block > 256 || (s->block % 32) != 0)
        return fail(MCGB_E_INVALID, "block size %u must be a multiple of 32 and <= 256", s->block);
    s->grid = (num_streams + s->block - 1) / s->block;
    s->lut_in_smem = (b->fp_lut && b->fp_lut_size > 0 && b->fp_lut_size <= 24576) ? 1 : 0;
    s->dyn_smem = s->lut_in_smem ? (size_t)b->fp_lut_size * sizeof(float) : 0;
    double d = deadline_s > 0.0 ? deadline_s : 300.0;
    s->deadline_ns = (uint64_t)(d * 1e9);
    (void)medium;
    (void)math;
    return MCGB_OK;
}

/* One device thread dumps n random numbers of one stream (RngKernel,
   xopto/mcbase/kernel/mcbase.template.c:1640-1646). */
__global__ void rng_dump_kernel(uint64_t x, uint32_t a, uint64_t n, float *out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (uint64_t i = 0; i < n; ++i) {
        x = (uint64_t)(uint32_t)x * (uint64_t)a + (x >> 32);
        out[i] = __uint2float_rn((uint32_t)x) * 2.3283064365386963e-10f;
    }
}

/* ScalarFillMcAccu (xopto/mcbase/kernel/mcbase.template.c:1740-1748) */
/* 16 independent FMA chains per thread, 8 unrolled steps per iteration;
   x -> x * 0.9999999 + 1e-7 stays near 1, so no chain overflows or goes
   subnormal. */
__global__ void __launch_bounds__(1024) fma_rate_kernel(uint32_t iters, float *out) {
    float a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = 1.0f + (float)(threadIdx.x + k) * 1e-6f;
    const float m = 0.9999999f, c = 1e-7f;
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
#pragma unroll
            for (int k = 0; k < 16; ++k) a[k] = fmaf(a[k], m, c);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += a[k];
    if (s == -1.0f) out[blockIdx.x] = s;
}

__global__ void fill_u64_kernel(uint64_t *p, uint64_t n, uint64_t v) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

}  // namespace

namespace mcgb_internal {
int set_error(int code, const char *msg) {
    g_last_error = msg;
    return code;
}
}  // namespace mcgb_internal

extern "C" {

const char *mcgb_last_error(void) { return g_last_error.c_str(); }

int mcgb_abi_version(void) { return MCGB_ABI_VERSION; }

int mcgb_sizeof(int kind) {
    switch (kind) {
        case 0: return (int)sizeof(McgbLayer);
        case 1: return (int)sizeof(McgbSource);
        case 2: return (int)sizeof(McgbDetector);
        case 3: return (int)sizeof(McgbFluence);
        case 4: return (int)sizeof(McgbTrace);
        case 5: return (int)sizeof(McgbMaterial);
        case 6: return (int)sizeof(McgbMcmlConfig);
        case 7: return (int)sizeof(McgbMcvoxConfig);
        case 8: return (int)sizeof(McgbBuffers);
        case 9: return (int)sizeof(McgbRunOptions);
        case 10: return (int)sizeof(McgbPf);
        case 11: return (int)sizeof(McgbBatchSim);
        case 12: return (int)sizeof(McgbBatchConfig);
        case 13: return (int)sizeof(McgbSurface);
        case 14: return (int)sizeof(McgbSamplingVolume);
        case 15: return (int)sizeof(McgbAdamwTensor);
        default: return -1;
    }
}

int mcgb_suggest_streams(int medium, int math, uint32_t block_size, uint32_t *streams) {
    if (!streams) return fail(MCGB_E_INVALID, "streams is NULL");
    int sms = 0, r = device_sm_count(&sms);
    if (r) return r;
    int bps = 0;
    unsigned block = block_size ? block_size : 128;
    cudaError_t e;
    if (math == MCGB_MATH_FAST)
        e = medium == 0 ? mcgb_fast::occupancy_mcml((int)block, 0, &bps)
                        : mcgb_fast::occupancy_mcvox((int)block, 0, &bps);
    else
        e = medium == 0 ? mcgb_exact::occupancy_mcml((int)block, 0, &bps)
                        : mcgb_exact::occupancy_mcvox((int)block, 0, &bps);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy");
    *streams = (uint32_t)sms * (uint32_t)bps * block;
    return MCGB_OK;
}

int mcgb_mcml_run(const McgbMcmlConfig *cfg, const McgbBuffers *buf, void *stream) {
    if (!cfg) return fail(MCGB_E_INVALID, "cfg is NULL");
    if (cfg->num_layers < 3 || cfg->num_layers > MCGB_MAX_LAYERS)
        return fail(MCGB_E_INVALID, "num_layers %u outside [3, %d]", cfg->num_layers, MCGB_MAX_LAYERS);
    McgbDetector dets[3] = {cfg->top, cfg->bottom, cfg->specular};
    int r = check_common(cfg->opt, cfg->pf_kind, cfg->num_packets, cfg->num_streams, cfg->source, dets,
                         cfg->fluence, cfg->trace, buf);
    if (r) return r;
    if (cfg->source.kind == MCGB_SRC_ISOTROPIC_VOXEL || cfg->source.kind == MCGB_SRC_ISOTROPIC_VOXELS)
        return fail(MCGB_E_UNSUPPORTED, "the voxel sources are implemented for voxelized media only");
    if ((cfg->source.kind == MCGB_SRC_UNIFORM_FIBER || cfg->source.kind == MCGB_SRC_LAMBERTIAN_FIBER ||
         cfg->source.kind == MCGB_SRC_UNIFORM_BEAM || cfg->source.kind == MCGB_SRC_UNIFORM_FIBER_LUT) &&
        !(cfg->source.direction[2] > 0.0f))
        return fail(MCGB_E_INVALID, "source: the z component of the direction must be positive");
    bool rectangular = cfg->source.kind == MCGB_SRC_UNIFORM_RECTANGULAR ||
                       cfg->source.kind == MCGB_SRC_LAMBERTIAN_RECTANGULAR ||
                       cfg->source.kind == MCGB_SRC_UNIFORM_RECTANGULAR_LUT;
    if ((cfg->source.kind == MCGB_SRC_ISOTROPIC_POINT || rectangular) &&
        (cfg->source.layer_index < 1 || cfg->source.layer_index > (int32_t)cfg->num_layers - 2))
        return fail(MCGB_E_INVALID, "source layer index %d outside the sample layers [1, %u]",
                    cfg->source.layer_index, cfg->num_layers - 2);
    if (rectangular) {
        if (cfg->specular.kind != MCGB_DET_NONE)
            return fail(MCGB_E_UNSUPPORTED, "rectangular sources take no specular detector "
                        "(the reference's launch code for them does not build with one)");
        if (!(cfg->source.angular >= 0.0f && cfg->source.angular <= 1.0f && cfg->source.clip >= 1.0f))
            return fail(MCGB_E_INVALID, "rectangular source: angular parameter %g, index %g",
                        (double)cfg->source.angular, (double)cfg->source.clip);
    }
    for (uint32_t i = 0; i < cfg->num_layers; ++i) {
        r = check_pf(cfg->pf_kind, cfg->layers[i].pf, buf, "layer", i);
        if (r) return r;
    }
    r = check_surface(cfg->surface_top, buf, "top");
    if (r) return r;
    r = check_surface(cfg->surface_bottom, buf, "bottom");
    if (r) return r;
    if (cfg->num_packets == 0) return MCGB_OK;
    LaunchShape s;
    r = make_shape(0, cfg->opt.math, cfg->opt.block_size, cfg->num_streams, buf, cfg->opt.deadline_s, &s);
    if (r) return r;
    cudaError_t e = (cfg->opt.math == MCGB_MATH_FAST)
                        ? mcgb_fast::launch_mcml(*cfg, *buf, (cudaStream_t)stream, s)
                        : mcgb_exact::launch_mcml(*cfg, *buf, (cudaStream_t)stream, s);
    if (e != cudaSuccess) return cuda_fail(e, "mcml launch");
    return MCGB_OK;
}

int mcgb_mcvox_run(const McgbMcvoxConfig *cfg, const McgbBuffers *buf, void *stream) {
    if (!cfg) return fail(MCGB_E_INVALID, "cfg is NULL");
    if (cfg->num_materials < 2 || cfg->num_materials > MCGB_MAX_MATERIALS)
        return fail(MCGB_E_INVALID, "num_materials %u outside [2, %d]", cfg->num_materials,
                    MCGB_MAX_MATERIALS);
    for (int k = 0; k < 3; ++k) {
        if (cfg->shape[k] <= 0) return fail(MCGB_E_INVALID, "voxel shape must be positive");
        if (!(cfg->voxel_size[k] > 0.0f)) return fail(MCGB_E_INVALID, "voxel size must be positive");
    }
    McgbDetector dets[3] = {cfg->top, cfg->bottom, cfg->specular};
    int r = check_common(cfg->opt, cfg->pf_kind, cfg->num_packets, cfg->num_streams, cfg->source, dets,
                         cfg->fluence, cfg->trace, buf);
    if (r) return r;
    if (cfg->top.kind >= MCGB_DET_TOTAL_LUT_PL || cfg->bottom.kind >= MCGB_DET_TOTAL_LUT_PL)
        return fail(MCGB_E_UNSUPPORTED, "the voxelized medium has TotalLut only among the look-up-table "
                    "detectors (xopto/mcvox/mcdetector)");
    if (cfg->source.kind == MCGB_SRC_UNIFORM_FIBER_NI || cfg->source.kind == MCGB_SRC_LAMBERTIAN_FIBER_NI ||
        (cfg->source.kind >= MCGB_SRC_UNIFORM_RECTANGULAR && cfg->source.kind != MCGB_SRC_ISOTROPIC_VOXELS &&
         cfg->source.kind != MCGB_SRC_UNIFORM_FIBER_LUT))
        return fail(MCGB_E_UNSUPPORTED, "source kind %d is implemented for layered media only",
                    cfg->source.kind);
    if (cfg->source.kind == MCGB_SRC_ISOTROPIC_VOXEL) {
        for (int k = 0; k < 3; ++k) {
            float v = cfg->source.direction[k];
            if (!(v >= 0.0f && v < (float)cfg->shape[k] && v == (float)(int)v))
                return fail(MCGB_E_INVALID, "voxel source index %g outside the grid", (double)v);
        }
    }
    if (!buf->voxels || !buf->materials) return fail(MCGB_E_INVALID, "voxel or material buffer is NULL");
    /* Voxel material indices are validated by the caller (uint8 < num_materials):
       the host wrapper checks the array before upload. */
    if (cfg->num_packets == 0) return MCGB_OK;
    LaunchShape s;
    r = make_shape(1, cfg->opt.math, cfg->opt.block_size, cfg->num_streams, buf, cfg->opt.deadline_s, &s);
    if (r) return r;
    cudaError_t e = (cfg->opt.math == MCGB_MATH_FAST)
                        ? mcgb_fast::launch_mcvox(*cfg, *buf, (cudaStream_t)stream, s)
                        : mcgb_exact::launch_mcvox(*cfg, *buf, (cudaStream_t)stream, s);
    if (e != cudaSuccess) return cuda_fail(e, "mcvox launch");
    return MCGB_OK;
}

int mcgb_check_counters(const uint64_t *dev_counters, void *stream, uint64_t *host_counters) {
    if (!dev_counters) return fail(MCGB_E_INVALID, "counters is NULL");
    uint64_t h[MCGB_NUM_COUNTERS];
    cudaError_t e = cudaMemcpyAsync(h, dev_counters, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "reading counters");
    if (host_counters) memcpy(host_counters, h, sizeof(h));
    uint64_t st = h[MCGB_CNT_STATUS];
    if (st & MCGB_STATUS_BAD_INDEX) return fail(MCGB_E_BAD_INDEX, "kernel reported an out-of-range index");
    if (st & MCGB_STATUS_TIMEOUT) return fail(MCGB_E_TIMEOUT, "run deadline expired before all packets finished");
    if (st & MCGB_STATUS_ABORTED) return fail(MCGB_E_TIMEOUT, "run aborted by the host");
    return MCGB_OK;
}

int mcgb_rng_dump(uint64_t x, uint32_t a, uint64_t n, float *dev_out, void *stream) {
    if (!dev_out && n) return fail(MCGB_E_INVALID, "output is NULL");
    if (n == 0) return MCGB_OK;
    rng_dump_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(x, a, n, dev_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MCGB_OK : cuda_fail(e, "rng dump launch");
}

int mcgb_fp32_fma_rate(uint32_t blocks, uint32_t threads, uint32_t iters, float *dev_out,
                       void *stream) {
    if (!dev_out) return fail(MCGB_E_INVALID, "output buffer is NULL");
    if (blocks == 0 || blocks > 65535u || threads == 0 || threads > 1024u || threads % 32u)
        return fail(MCGB_E_INVALID, "fma probe: %u blocks of %u threads", blocks, threads);
    fma_rate_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, dev_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MCGB_OK : cuda_fail(e, "fma probe launch");
}

int mcgb_fill_u64(uint64_t *dev, uint64_t n, uint64_t value, void *stream) {
    if (n == 0) return MCGB_OK;
    if (!dev) return fail(MCGB_E_INVALID, "buffer is NULL");
    unsigned blocks = (unsigned)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    fill_u64_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(dev, n, value);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MCGB_OK : cuda_fail(e, "fill launch");
}

int mcgb_batched_work_size(uint32_t num_sims, uint64_t *bytes) {
    if (!bytes) return fail(MCGB_E_INVALID, "bytes is NULL");
    *bytes = batch_work_bytes(num_sims);
    return MCGB_OK;
}

int mcgb_batched_occupancy(uint32_t block_size, int math, uint32_t *blocks_per_sm) {
    if (!blocks_per_sm) return fail(MCGB_E_INVALID, "blocks_per_sm is NULL");
    int n = 0;
    cudaError_t e = (math == MCGB_MATH_FAST) ? mcgb_fast_batch::batched_occupancy((int)block_size, &n)
                                             : mcgb_exact_batch::batched_occupancy((int)block_size, &n);
    if (e != cudaSuccess) return cuda_fail(e, "batched occupancy");
    *blocks_per_sm = (uint32_t)n;
    return MCGB_OK;
}

int mcgb_batched_run(const McgbBatchConfig *cfg, const McgbBatchSim *dev_sims,
                     const uint32_t *dev_multipliers, uint64_t *dev_tally, void *dev_work,
                     uint64_t *dev_counters, void *stream) {
    if (!cfg) return fail(MCGB_E_INVALID, "cfg is NULL");
    if (cfg->num_sims == 0) return MCGB_OK;
    if (cfg->num_sims > (1u << 24)) return fail(MCGB_E_SIZE, "at most 2^24 simulations per batch");
    if (!dev_sims || !dev_multipliers || !dev_tally || !dev_work || !dev_counters)
        return fail(MCGB_E_INVALID, "NULL device buffer");
    if (cfg->num_bins == 0) return fail(MCGB_E_INVALID, "num_bins must be positive");
    if (cfg->num_multipliers < 1) return fail(MCGB_E_INVALID, "no RNG multipliers");
    if (cfg->packets_per_item < 32) return fail(MCGB_E_INVALID, "packets_per_item must be >= 32");
    if (cfg->math != MCGB_MATH_EXACT && cfg->math != MCGB_MATH_FAST)
        return fail(MCGB_E_INVALID, "unknown math mode %d", cfg->math);
    if (!(cfg->inv_dr >= 0.0f)) return fail(MCGB_E_INVALID, "inv_dr must be non-negative");
    unsigned block = cfg->block_size ? cfg->block_size : 128;
    if (block > 256 || block % 32) return fail(MCGB_E_INVALID, "block size must be a multiple of 32, <= 256");
    if (((uintptr_t)dev_work) % 16) return fail(MCGB_E_INVALID, "work buffer must be 16-byte aligned");
    int sms = 0, r = device_sm_count(&sms);
    if (r) return r;
    uint32_t bps = cfg->blocks_per_sm;
    if (!bps) {
        r = mcgb_batched_occupancy(block, cfg->math, &bps);
        if (r) return r;
        if (!bps) return fail(MCGB_E_INVALID, "block size %u does not fit an SM", block);
    }
    unsigned grid = (unsigned)sms * bps;
    double d = cfg->deadline_s > 0.0 ? cfg->deadline_s : 300.0;
    uint64_t deadline = (uint64_t)(d * 1e9);
    cudaError_t e = (cfg->math == MCGB_MATH_FAST)
        ? mcgb_fast_batch::launch_batched(*cfg, dev_sims, dev_multipliers, dev_tally, dev_work,
                                          dev_counters, (cudaStream_t)stream, grid, block, deadline)
        : mcgb_exact_batch::launch_batched(*cfg, dev_sims, dev_multipliers, dev_tally, dev_work,
                                           dev_counters, (cudaStream_t)stream, grid, block, deadline);
    if (e != cudaSuccess) return cuda_fail(e, "batched launch");
    return MCGB_OK;
}

int mcgb_sampling_volume(const McgbSamplingVolume *sv, const float *dev_trace,
                         uint64_t trace_floats, const int32_t *dev_counts,
                         uint64_t *dev_accu, uint64_t accu_size, uint64_t *dev_total_weight,
                         uint64_t *dev_counters, void *stream) {
    if (!sv) return fail(MCGB_E_INVALID, "sampling volume is NULL");
    uint64_t voxels = 1;
    for (int i = 0; i < 3; ++i) {
        if (sv->shape[i] == 0 || sv->shape[i] > 2147483647u)
            return fail(MCGB_E_INVALID, "sampling volume: shape[%d] = %u outside [1, 2^31 - 1]", i,
                        sv->shape[i]);
        if (!std::isfinite(sv->voxel_size[i]) || sv->voxel_size[i] == 0.0f ||
            !std::isfinite(sv->top_left[i]))
            return fail(MCGB_E_INVALID, "sampling volume: axis %d has corner %g and voxel size %g", i,
                        (double)sv->top_left[i], (double)sv->voxel_size[i]);
        voxels *= sv->shape[i];
    }
    if (voxels > (1ull << 40)) return fail(MCGB_E_SIZE, "sampling volume: %llu voxels", (unsigned long long)voxels);
    if (sv->offset > accu_size || voxels > accu_size - sv->offset)
        return fail(MCGB_E_SIZE, "sampling volume: voxels [%llu, +%llu) beyond the accumulator (%llu)",
                    (unsigned long long)sv->offset, (unsigned long long)voxels,
                    (unsigned long long)accu_size);
    if (sv->num_packets == 0) return MCGB_OK;
    if (sv->max_events == 0) return fail(MCGB_E_INVALID, "sampling volume: max_events is 0");
    if (sv->num_packets > (1ull << 40) / sv->max_events)
        return fail(MCGB_E_SIZE, "sampling volume: %llu packets of %u events",
                    (unsigned long long)sv->num_packets, sv->max_events);
    uint64_t need = sv->num_packets * sv->max_events * MCGB_TRACE_ENTRY_LEN;
    if (trace_floats < need)
        return fail(MCGB_E_SIZE, "sampling volume: trace of %llu floats, %llu needed",
                    (unsigned long long)trace_floats, (unsigned long long)need);
    if (!dev_trace || !dev_counts || !dev_accu || !dev_total_weight)
        return fail(MCGB_E_INVALID, "sampling volume: NULL trace, count, accumulator or weight buffer");
    if (reinterpret_cast<uintptr_t>(dev_trace) % 16)
        return fail(MCGB_E_INVALID, "sampling volume: trace buffer not 16-byte aligned");
    cudaError_t e = mcgb_sv::launch(*sv, dev_trace, dev_counts, dev_accu, dev_total_weight,
                                    dev_counters, (cudaStream_t)stream);
    return e == cudaSuccess ? MCGB_OK : cuda_fail(e, "sampling volume launch");
}

int mcgb_reduce_tallies(uint64_t *host_dst, const uint64_t *host_src, uint64_t n) {
    if (n && (!host_dst || !host_src)) return fail(MCGB_E_INVALID, "NULL tally array");
    for (uint64_t i = 0; i < n; ++i) host_dst[i] += host_src[i];
    return MCGB_OK;
}

}  // extern "C"
