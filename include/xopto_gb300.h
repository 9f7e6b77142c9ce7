/*
 * xopto_gb300.h - C ABI of libxopto_gb300.so, the GB300 (sm_103a) Monte Carlo
 * photon-packet transport engine for layered (mcml) and voxelized (mcvox)
 * turbid media.
 *
 * Reference interfaces replaced (paths inside the PyXOpto project):
 *   mcgb_mcml_run      xopto/mcml/kernel/mcml.template.c:346  McKernel (mcml),
 *                      launched by xopto/mcml/mc.py:922-953
 *   mcgb_mcvox_run     xopto/mcvox/kernel/mcvox.template.c:548 McKernel (mcvox),
 *                      launched by xopto/mcvox/mc.py:968
 *   mcgb_rng_dump      xopto/mcbase/kernel/mcbase.template.c:1640 RngKernel,
 *                      launched by xopto/mcml/mc.py:1320-1362 (Mc.rng_test)
 *   mcgb_rng_init      xopto/src/rng/rng.cpp:64 init_RNG and
 *                      xopto/cl/clrng.py:184 _rng_init
 *   mcgb_rng_safeprimes xopto/src/rng/find_primes.c:40 (safe-prime multipliers,
 *                      table xopto/data/primes/safeprimes_base32_500k.npz)
 *   mcgb_sizeof        xopto/mcml/kernel/mcml.template.c:827 sizeof_datatypes
 *   mcgb_fill_u64      xopto/mcbase/kernel/mcbase.template.c:1740 ScalarFillMcAccu
 *   mcgb_batched_run   (new) batched persistent engine; replaces the sequential
 *                      loop xopto/mcml/mcrun/helper.py:640-686
 *   mcgb_mlp_*         (new) BF16 surrogate kernels; the reference trains its
 *                      networks with TensorFlow (xopto/util/regression/ann.py)
 *
 * Conventions
 *   - Plain pointers and sizes only.  "dev" pointers are device memory owned
 *     by the caller (cudaMalloc or a torch tensor); the library never frees
 *     caller memory.  "host" pointers are host memory.
 *   - Every entry point returns 0 (MCGB_OK) on success or a negative
 *     MCGB_E_* code.  mcgb_last_error() returns a text description of the
 *     last failure on the calling host thread.  No C++ exception crosses the
 *     ABI.
 *   - Launch functions enqueue work on the caller's stream (a cudaStream_t
 *     passed as void*, NULL = legacy default stream) and return without
 *     waiting; the caller synchronizes before reading results, as the
 *     reference waits on its OpenCL event (xopto/mcml/mc.py:953).
 *   - Units are SI (m, 1/m), as in the reference (xopto/mcml/mclayer/layer.py).
 *   - Tallies are 64-bit unsigned fixed-point integers: each deposit adds
 *     (uint32_t)(w*K + 0.5f) with K = MCGB_ACCU_K (the reference's
 *     MC_INT_ACCUMULATOR_K, xopto/mcbase/kernel/mcbase.template.h:237), so
 *     totals do not depend on the order of the deposits.
 *
 * Packet-to-stream mapping: a run of N packets on T random-number streams
 * gives stream t the packets t, t+T, t+2T, ... < N, each simulated to
 * completion in order with stream t's multiply-with-carry generator.  Results
 * are therefore bit-reproducible for a given seed table, T and math mode.
 */
#ifndef XOPTO_GB300_H
#define XOPTO_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCGB_ABI_VERSION 3

/* Fixed-point weight scale of the integer accumulators. */
#define MCGB_ACCU_K 8388607
/* Largest layer stack (including the two surrounding half-spaces). */
#define MCGB_MAX_LAYERS 64
/* Largest material table of a voxelized sample (voxels are uint8 indices). */
#define MCGB_MAX_MATERIALS 256
/* Floats in one trace event (xopto/mcbase/mctrace.py TRACE_ENTRY_LEN). */
#define MCGB_TRACE_ENTRY_LEN 8
/* Voxel crossings after which a sampling-volume walk of one packet stops. */
#define MCGB_SV_MAX_CROSSINGS (1u << 26)

/* ---------------------------------------------------------------- errors */
enum {
    MCGB_OK = 0,
    MCGB_E_INVALID = -1,     /* invalid argument or configuration        */
    MCGB_E_SIZE = -2,        /* buffer too small / size limit exceeded   */
    MCGB_E_CUDA = -3,        /* CUDA runtime error                       */
    MCGB_E_TIMEOUT = -4,     /* device deadline expired, run incomplete  */
    MCGB_E_BAD_INDEX = -5,   /* kernel caught an out-of-range index      */
    MCGB_E_UNSUPPORTED = -6  /* feature not built into this library      */
};

/* Status bits written by the kernels into counters[MCGB_CNT_STATUS]. */
#define MCGB_STATUS_TIMEOUT    0x1u
#define MCGB_STATUS_BAD_INDEX  0x2u
#define MCGB_STATUS_STEP_LIMIT 0x4u
#define MCGB_STATUS_ABORTED    0x8u

/* Device counter block (uint64_t[MCGB_NUM_COUNTERS], caller-owned). */
enum {
    MCGB_CNT_PACKETS = 0,    /* packets completed                        */
    MCGB_CNT_STEPS = 1,      /* interaction steps (loop iterations)      */
    MCGB_CNT_STATUS = 2,     /* OR of MCGB_STATUS_* bits                 */
    MCGB_CNT_THREADS = 3,    /* threads that simulated >= 1 packet       */
    MCGB_CNT_ABORT = 4,      /* set nonzero by the host to stop a run    */
    MCGB_CNT_QUEUE = 5,      /* work queue of dynamic scheduling (zero it) */
    MCGB_NUM_COUNTERS = 8
};

/* ----------------------------------------------------------- enumerations */
enum { MCGB_METHOD_ALBEDO_WEIGHT = 0,       /* MC_METHOD 0 (default)      */
       MCGB_METHOD_ALBEDO_REJECTION = 1,    /* MC_METHOD 1                */
       MCGB_METHOD_MICROSCOPIC_BEER_LAMBERT = 2 };
enum { MCGB_PF_HG = 0, MCGB_PF_GK = 1, MCGB_PF_LUT = 2,
       MCGB_PF_EXT = 3 };                   /* the analytic samplers below */
/* McgbPf.ext_kind of an MCGB_PF_EXT phase function */
enum { MCGB_PF_EXT_HG2 = 0,                /* xopto/mcbase/mcpf/hg2.py:102-130 */
       MCGB_PF_EXT_MHG = 1,                /* xopto/mcbase/mcpf/mhg.py:87-109  */
       MCGB_PF_EXT_PC = 2,                 /* xopto/mcbase/mcpf/pc.py:80-92    */
       MCGB_PF_EXT_MPC = 3,                /* xopto/mcbase/mcpf/mpc.py:88-106  */
       MCGB_PF_EXT_MGK = 4,                /* xopto/mcbase/mcpf/mgk.py:110-140 */
       MCGB_PF_EXT_GK2 = 5,                /* xopto/mcbase/mcpf/gk2.py:119-159 */
       MCGB_PF_EXT_HGA = 6,                /* xopto/mcbase/mcpf/hga.py:82-99   */
       MCGB_PF_EXT_HGDIR = 7 };            /* xopto/mcbase/mcpf/hgdir.py:100-120 */
/* Parameters of the analytic kinds: McgbPf.p holds them in the order of the
   reference's packed struct (Hg2: g1, g2, b; MHg: g, b; Pc: n; MPc: n, b;
   MGk: g, b, inv_a, a1, a2; HgDir: direction x, y, z, g, p).  Gk2 and Hga
   keep theirs in the float LUT at McgbPf.lut_offset: Gk2 the 11 floats
   (g, a, inv_a, a1, a2) of each term and b; Hga the 3x3 anisotropy tensor,
   row major. */
#define MCGB_PF_GK2_FLOATS 11u
#define MCGB_PF_HGA_FLOATS 9u
enum {
    MCGB_SRC_LINE = 0,
    MCGB_SRC_GAUSSIAN_BEAM = 1,
    MCGB_SRC_UNIFORM_FIBER_NI = 2,
    MCGB_SRC_LAMBERTIAN_FIBER_NI = 3,
    MCGB_SRC_UNIFORM_FIBER = 4,
    MCGB_SRC_LAMBERTIAN_FIBER = 5,
    MCGB_SRC_UNIFORM_BEAM = 6,
    MCGB_SRC_ISOTROPIC_POINT = 7,
    MCGB_SRC_ISOTROPIC_VOXEL = 8,
    MCGB_SRC_UNIFORM_RECTANGULAR = 9,
    MCGB_SRC_LAMBERTIAN_RECTANGULAR = 10,
    MCGB_SRC_UNIFORM_FIBER_LUT_NI = 11,
    MCGB_SRC_UNIFORM_FIBER_LUT = 12,
    MCGB_SRC_UNIFORM_RECTANGULAR_LUT = 13,
    MCGB_SRC_ISOTROPIC_VOXELS = 14
};
enum { MCGB_DET_NONE = 0, MCGB_DET_TOTAL = 1, MCGB_DET_RADIAL = 2, MCGB_DET_RADIAL_PL = 3,
       MCGB_DET_TOTAL_PL = 4, MCGB_DET_CARTESIAN = 5, MCGB_DET_CARTESIAN_PL = 6,
       MCGB_DET_SYMMETRIC_X = 7, MCGB_DET_LINEAR_ARRAY = 8, MCGB_DET_SIX_AROUND_ONE = 9,
       MCGB_DET_FIBER_ARRAY = 10, MCGB_DET_LINEAR_ARRAY_PL = 11, MCGB_DET_SIX_AROUND_ONE_PL = 12,
       MCGB_DET_FIBER_ARRAY_PL = 13, MCGB_DET_TOTAL_LUT = 14, MCGB_DET_TOTAL_LUT_PL = 15,
       MCGB_DET_FIBER_LUT_ARRAY = 16 };
#define MCGB_DET_FIBER_FLOATS 13            /* floats per FIBER_ARRAY fibre    */
#define MCGB_DET_LUT_FIBER_FLOATS 16        /* floats per FIBER_LUT_ARRAY fibre */
enum { MCGB_FLUENCE_NONE = 0, MCGB_FLUENCE_DEPOSITION = 1, MCGB_FLUENCE_RATE = 2 };
/* Trace flags (xopto/mcbase/mctrace.py TRACE_START/END/ALL). */
enum { MCGB_TRACE_NONE = 0, MCGB_TRACE_START = 1, MCGB_TRACE_END = 2, MCGB_TRACE_ALL = 7 };
/* Math mode: EXACT evaluates log/sin/cos/pow/exp with the library's own
   portable single-precision routines and IEEE +,-,*,/,sqrt without FMA
   contraction, so GPU and CPU produce identical bits.  FAST uses the GPU's
   special-function units (the reference's MC_USE_NATIVE_MATH). */
enum { MCGB_MATH_EXACT = 0, MCGB_MATH_FAST = 1 };
/* Packet scheduling.  STATIC: thread t owns random-number stream t (state
   rng_x[t], multiplier rng_a[t]) and simulates packets t, t+T, t+2T, ...
   (the reference's per-thread streams).  DYNAMIC: persistent warps take
   packets from a device work queue (counters[MCGB_CNT_QUEUE], zeroed by the
   caller) and refill idle lanes packet by packet; packet p simulates on
   its own MWC stream derived from (seed, packet_offset + p) with a
   multiplier from rng_a[0 .. num_streams) (batch_rng.h); rng_x is unused.
   Both are bit-reproducible; DYNAMIC keeps every lane busy until the last
   packets. */
enum { MCGB_SCHED_STATIC = 0, MCGB_SCHED_DYNAMIC = 1 };

/* ------------------------------------------------------------ POD structs */
/* Scattering phase function of one layer/material.
   Hg:  p[0]=g                      (xopto/mcbase/mcpf/hg.py:80-95)
   Gk:  p[0..4]=g, a, inv_a, a1, a2 (xopto/mcbase/mcpf/gk.py:102-124,153-178)
   Lut: p[0..2]=a, b, c; lut_offset, lut_size (xopto/mcbase/mcpf/lut.py:125-155)
   Ext: ext_kind selects the sampler;
        Hg2 p[0..2]=g1, g2, b; MHg p[0..1]=g, beta; Pc p[0]=n; MPc p[0..1]=n, beta;
        MGk p[0..4]=g, beta, inv_a, a1, a2 (a == 0 is inv_a == 0 with g != 0) */
typedef struct McgbPf {
    float p[5];
    uint32_t lut_offset;
    uint32_t lut_size;
    uint32_t ext_kind;                      /* MCGB_PF_EXT_* (Ext only)         */
} McgbPf;                                   /* 32 bytes */

/* One layer (xopto/mcml/mclayer/layer.py:40-72 ClLayer). */
typedef struct McgbLayer {
    float thickness, top, bottom, n;
    float cos_critical_top, cos_critical_bottom;
    float mus, mua, inv_mut, mua_inv_mut;
    McgbPf pf;
} McgbLayer;                                /* 72 bytes */

/* One material of a voxelized sample (xopto/mcbase/mcmaterial.py:54-61). */
typedef struct McgbMaterial {
    float n, mus, mua, inv_mut, mua_inv_mut;
    float reserved[3];
    McgbPf pf;
} McgbMaterial;                             /* 64 bytes */

/* Photon packet source.
   Line (xopto/mcml/mcsource/line.py:56-62,181-228): position on the sample
     surface, direction = direction in the sample, direction_reflected,
     reflectance = specular reflectance.
   GaussianBeam mcml (xopto/mcml/mcsource/gaussianbeam.py:119-170,300-362):
     transformation, position, direction (refracted), sigma, clip,
     reflectance.
   GaussianBeam mcvox (xopto/mcvox/mcsource/gaussianbeam.py:112-190):
     transformation, position, direction (in the surrounding medium), sigma,
     clip.
   Fibre sources, layered media only (xopto/mcml/mcsource/fiberni.py,
   fiber.py): position = centre of the fibre core on the sample surface,
   sigma[0] = core radius, clip = refractive index of the core, and
     UniformFiberNI (fiberni.py:246-290,383-412): sigma[1] = cosine of the
       acceptance angle in air, sqrt(1 - NA^2);
     LambertianFiberNI (fiberni.py:485-534,562-573): sigma[1] = NA;
     UniformFiber (fiber.py:267-330,429-470): sigma[1] = sqrt(1 - NA^2),
       direction = fibre axis, transformation = rotation of the z axis onto
       it;
     LambertianFiber (fiber.py:576-640,660-681): sigma[1] = NA, direction
       and transformation as UniformFiber.
   UniformBeam mcml (xopto/mcml/mcsource/uniformbeam.py:107-146,243-292):
     elliptical flat-top beam; transformation, position on the surface,
     direction (refracted), sigma = radii along x and y, reflectance.
   IsotropicPoint mcml (xopto/mcml/mcsource/point.py:76-128,188-226):
     position (above the sample: z <= 0, or inside it) and layer_index of
     the layer that holds it (1 for a point above the sample).
   Voxelized media (xopto/mcvox/mcsource): UniformBeam (uniformbeam.py:
     104-186) and the tilted fibres UniformFiber / LambertianFiber
     (fiber.py:257-352,603-700) take transformation, position (anywhere;
     moved onto the voxel box along the direction), direction (in the
     surrounding medium), sigma (beam radii; fibre core radius and
     sqrt(1 - NA^2) or NA) and clip (fibre core index); IsotropicPoint
     (point.py:74-140) takes position; IsotropicVoxel (voxel.py:78-107) takes
     the voxel index as floats in direction and the voxel centre in position
     (the centre of the rmax sphere, mcvox.template.c:585,983).
   UniformRectangular / LambertianRectangular, layered media only
     (xopto/mcml/mcsource/rectangular.py:85-140,363-413): position = centre
     (z = 0 for a source on the surface), sigma = width (x) and height (y),
     clip = refractive index of the source, angular = cosine of the maximum
     emission angle in air (uniform) or NA (Lambertian), layer_index = the
     layer that holds the source.  The reference's rectangular sources do not
     build with a specular detector (their launch reads a reflectance field
     the source lacks), so that combination is rejected.
   Emission look-up-table sources, layered media only: the cosine of the
     emission angle in air is drawn from lut_size floats of the float table
     at lut_offset (EmissionLut, sampled by the reference's
     fp_linear_lut_rel_sample, xopto/mcbase/kernel/mcbase.template.h:2507-2520).
     UniformFiberLutNI (xopto/mcml/mcsource/fiberni.py:581-700) takes the
     UniformFiberNI fields; UniformFiberLut (fiber.py:690-830) the
     UniformFiber fields, and unlike UniformFiber it refracts the launch
     direction into the sample; UniformRectangularLut (rectangular.py:530-700)
     the rectangular fields without angular.
   IsotropicVoxels, voxelized media only (xopto/mcvox/mcsource/voxel.py:
     195-380): lut_size voxels of 4 floats (weight, x, y, z voxel index) in
     the float table at lut_offset; a packet starts in one of them, chosen
     uniformly, with that weight; position = centre of the mean voxel index. */
typedef struct McgbSource {
    int32_t kind;
    float position[3];
    float direction[3];
    float direction_reflected[3];
    float reflectance;
    float transformation[9];                /* row-major a_11 .. a_33 */
    float sigma[2];
    float clip;
    int32_t layer_index;                    /* IsotropicPoint, rectangular     */
    float angular;                          /* rectangular: cos_min or NA      */
    uint32_t lut_offset;                    /* emission LUT sources            */
    uint32_t lut_size;
} McgbSource;                               /* 108 bytes */

/* Surface detector (xopto/mcml/mcdetector/radial.py:66-75,117-150;
   total.py:52-56,86-108; radialpl.py:138-179,343-378; totalpl.py:107-135;
   cartesian.py:124-157,340-372; cartesianpl.py:150-190; symmetric.py:124-156,
   260-285).
   Total: one bin.  Radial: n radial bins (r_min, inv_dr, log_scale).
   TotalPl: n_pl optical path-length bins.  RadialPl: n_pl x n bins, path
   length first.  Cartesian: n_y x n bins, x axis (r_min, inv_dr, n) and y
   axis (y_min, inv_dy, n_y).  CartesianPl: n_pl x n_y x n bins.  SymmetricX:
   2n bins symmetric about x = position[0], half axis offset r_min, 1/step
   inv_dr, log_scale.  Indices outside an axis are clipped into its first or
   last bin; the path-length kinds need
   McgbRunOptions.track_optical_pathlength.
   Fibre-probe detectors (xopto/mcml/mcdetector/probe): one bin per fibre
   (n fibres; the _PL kinds n_pl x n, path length first) and a float table
   in McgbBuffers.fp_lut from table_offset:
     LINEAR_ARRAY (lineararray.py:103-162,341-380): transformation (9),
       first fibre position (2), fibre step (2), core r^2, acceptance cosine;
     SIX_AROUND_ONE (sixaroundone.py:103-184,346-386; n = 7):
       transformation (9), position (2), core r^2, core spacing, acceptance
       cosine;
     FIBER_ARRAY (fiberarray.py:103-162,270-312): per fibre transformation
       (9), position (2), core r^2, acceptance cosine.  Top and bottom slots
       only.
   Collection look-up-table detectors: the deposit is the weight times a
   sensitivity read from a CollectionLut at |cos| of the exit direction, by
   the reference's fp_linear_lut_sample
   (xopto/mcbase/kernel/mcbase.template.h:2522-2535; 0 outside the table):
     TOTAL_LUT (total.py:240-330) and TOTAL_LUT_PL (totalpl.py, TotalLutPl):
       direction, LUT first position in r_min, 1/span in inv_dr, size in n_y,
       offset in table_offset; n = 1 (TOTAL_LUT_PL: n_pl bins);
     FIBER_LUT_ARRAY (probe/fiberlutarray.py:30-200,290-324): n fibres, per
       fibre transformation (9), position (2), core r^2, LUT first position,
       1/span, and the LUT size and offset as uint32 bit patterns. */
typedef struct McgbDetector {
    int32_t kind;
    float direction[3];
    float position[2];
    float r_min, inv_dr, cos_min;
    uint32_t n;                             /* radial / x bins                 */
    int32_t log_scale;                      /* radial / x axis in log scale    */
    int32_t pl_log_scale;                   /* path-length axis in log scale   */
    uint64_t offset;                        /* first accumulator               */
    float pl_min, inv_dpl;                  /* path-length axis start, 1/step  */
    uint32_t n_pl;                          /* path-length bins                */
    uint32_t table_offset;                  /* fibre probes: first float       */
    float y_min, inv_dy;                    /* Cartesian y axis start, 1/step  */
    uint32_t n_y;                           /* Cartesian y bins                */
    uint32_t reserved2;
} McgbDetector;                             /* 88 bytes */

/* Cartesian fluence (xopto/mcbase/mcfluence/fluence.py:56-62,103-143). */
typedef struct McgbFluence {
    int32_t kind;
    float inv_step[3];
    float top_left[3];
    uint32_t shape[3];
    int32_t k;
    uint32_t reserved;
    uint64_t offset;                        /* first accumulator */
} McgbFluence;                              /* 56 bytes */

/* Packet trace (xopto/mcbase/mctrace.py:541-583). */
typedef struct McgbTrace {
    int32_t flags;                          /* MCGB_TRACE_* */
    uint32_t max_events;
    uint32_t event_mask;                    /* 0 = record every event */
    uint32_t reserved;
    uint64_t data_offset;                   /* in the float buffer */
    uint64_t count_offset;                  /* in the int buffer   */
} McgbTrace;                                /* 32 bytes */

/* Sampling volume of a set of packet traces (replaces the reference's
   SamplingVolume kernel arguments: ClSamplingVolume,
   xopto/mcbase/mcsv.py:30-95, and the McTrace fields that kernel reads,
   xopto/mcbase/kernel/mcsv.template.c:236-262).  The traces are
   num_packets records of max_events events of MCGB_TRACE_ENTRY_LEN floats
   (x, y, z, px, py, pz, w, pl) plus one int32 event count per packet. */
typedef struct McgbSamplingVolume {
    float top_left[3];                      /* x, y, z of the first voxel's corner */
    float voxel_size[3];
    uint32_t shape[3];                      /* voxels along x, y, z            */
    float multiplier;                       /* applied to weight x path length */
    uint64_t offset;                        /* first voxel in the accumulator  */
    int32_t k;                              /* float to integer weight factor  */
    uint32_t max_events;                    /* trace length per packet         */
    uint64_t num_packets;                   /* traces to process               */
} McgbSamplingVolume;                       /* 64 bytes */

/* Options shared by both media. */
typedef struct McgbRunOptions {
    int32_t method;                         /* MCGB_METHOD_*                   */
    int32_t math;                           /* MCGB_MATH_*                     */
    int32_t use_lottery;                    /* MC_USE_LOTTERY (default 1)      */
    float packet_weight_min;                /* MC_PACKET_WEIGHT_MIN (1e-4)     */
    float lottery_chance;                   /* MC_PACKET_LOTTERY_CHANCE (0.1)  */
    float rmax;                             /* Mc.rmax (inf = no limit)        */
    int32_t track_optical_pathlength;       /* MC_TRACK_OPTICAL_PATHLENGTH     */
    uint32_t block_size;                    /* threads per block (0 = auto);
                                               STATIC scheduling only, the
                                               DYNAMIC kernels use 128         */
    uint64_t max_steps_per_packet;          /* 0 = unlimited (2^32 - 1 at most) */
    double deadline_s;                      /* device wall-clock limit, 0=300s */
    int32_t scheduling;                     /* MCGB_SCHED_*                    */
    uint32_t packets_per_item;              /* DYNAMIC: packets a warp takes
                                               from the queue at a time, 1-128
                                               (0 = chosen from the packet
                                               count and the grid)             */
    uint64_t seed;                          /* DYNAMIC: stream derivation seed */
    uint64_t packet_offset;                 /* DYNAMIC: index of packet 0      */
} McgbRunOptions;

/* Layout of the top or bottom sample surface (xopto/mcml/mcsurface): the
   handler runs where a packet meets that surface and may change the
   refractive index and critical cosine of the boundary or reflect the
   packet itself.  The parameters are n floats of the float table
   (McgbBuffers.fp_lut) from table_offset on:
     LAMBERTIAN (lambertian.py:70-106): reflectance, specular fraction;
     LINEAR_ARRAY (probe/lineararray.py:167-239,492-552): transformation (9),
       probe position (2), first fibre position (2), fibre step (2), core r^2,
       core n, core critical cosine, cladding r^2, cladding n, cladding
       critical cosine, probe r^2, probe reflectivity, cutout transformation
       (4), cutout half width, cutout half height, cutout n, cutout critical
       cosine; n_fibers = fibres;
     SIX_AROUND_ONE (probe/sixaroundone.py:158-262,495-545): transformation
       (9), position (2), core spacing, core r^2, core n, core critical cosine,
       cladding r^2, cladding n, cladding critical cosine, cutout r^2, cutout
       n, cutout critical cosine, probe r^2, probe reflectivity;
     FIBER_ARRAY (probe/fiberarray.py:136-187,330-390): probe position (2),
       probe r^2, probe reflectivity, then per fibre: transformation (9),
       position (2), cladding r^2, cladding n, cladding critical cosine, core
       r^2, core n, core critical cosine; n_fibers = fibres. */
enum {
    MCGB_SURFACE_NONE = 0,
    MCGB_SURFACE_LAMBERTIAN = 1,
    MCGB_SURFACE_LINEAR_ARRAY = 2,
    MCGB_SURFACE_SIX_AROUND_ONE = 3,
    MCGB_SURFACE_FIBER_ARRAY = 4
};
#define MCGB_SURFACE_FIBER_FLOATS 17        /* floats per FIBER_ARRAY fibre    */

typedef struct McgbSurface {
    int32_t kind;                           /* MCGB_SURFACE_*                  */
    uint32_t n_fibers;
    uint32_t table_offset;                  /* first float in the float table  */
    uint32_t table_size;                    /* floats                          */
} McgbSurface;                              /* 16 bytes */

/* Layered medium run (the reference's McKernel arguments for mcml). */
typedef struct McgbMcmlConfig {
    uint64_t num_packets;
    uint32_t num_streams;                   /* RNG streams = device threads    */
    int32_t pf_kind;                        /* MCGB_PF_*                       */
    uint32_t num_layers;
    uint32_t reserved;
    McgbRunOptions opt;
    McgbSource source;
    McgbDetector top, bottom, specular;
    McgbFluence fluence;
    McgbTrace trace;
    McgbSurface surface_top, surface_bottom;
    McgbLayer layers[MCGB_MAX_LAYERS];
} McgbMcmlConfig;

/* Voxelized medium run (the reference's McKernel arguments for mcvox,
   xopto/mcvox/mcgeometry/voxel.py:88-165 McVoxelConfig).  Material 0 is the
   surrounding medium (xopto/mcvox/kernel/mcvox.template.h:772-779). */
typedef struct McgbMcvoxConfig {
    uint64_t num_packets;
    uint32_t num_streams;
    int32_t pf_kind;
    uint32_t num_materials;
    uint32_t reserved;
    McgbRunOptions opt;
    float top_left[3];
    float bottom_right[3];
    float voxel_size[3];
    int32_t shape[3];
    McgbSource source;
    McgbDetector top, bottom, specular;
    McgbFluence fluence;
    McgbTrace trace;
} McgbMcvoxConfig;

/* Device buffers of one run (all caller-owned device memory). */
typedef struct McgbBuffers {
    uint64_t *rng_x;                /* [num_streams] mutable MWC states      */
    const uint32_t *rng_a;          /* [num_streams] MWC multipliers         */
    uint64_t *accumulator;          /* detector + fluence tallies            */
    uint64_t accumulator_size;
    float *float_buffer;            /* trace events                          */
    uint64_t float_size;
    int32_t *int_buffer;            /* trace event counts                    */
    uint64_t int_size;
    const float *fp_lut;            /* phase-function lookup tables          */
    uint64_t fp_lut_size;
    const uint8_t *voxels;          /* mcvox: material index per voxel,
                                       flat index (z*ny + y)*nx + x          */
    const McgbMaterial *materials;  /* mcvox: [num_materials]                */
    const uint8_t *voxel_radius;    /* mcvox, FAST math: homogeneous-cube
                                       radius per voxel (mcgb_voxel_radius),
                                       or NULL to stop at every voxel wall   */
    uint64_t *counters;             /* [MCGB_NUM_COUNTERS]                   */
} McgbBuffers;

/* ------------------------------------------------------------ entry points */
const char *mcgb_last_error(void);
int mcgb_abi_version(void);
/* Size of one of the POD structs above, for host/device layout checks
   (replaces the reference's sizeof_datatypes kernel).  kind: 0 McgbLayer,
   1 McgbSource, 2 McgbDetector, 3 McgbFluence, 4 McgbTrace, 5 McgbMaterial,
   6 McgbMcmlConfig, 7 McgbMcvoxConfig, 8 McgbBuffers, 9 McgbRunOptions,
   10 McgbPf, 11 McgbBatchSim, 12 McgbBatchConfig, 13 McgbSurface,
   14 McgbSamplingVolume, 15 McgbAdamwTensor.  Returns -1 for an unknown
   kind. */
int mcgb_sizeof(int kind);

/* Number of streams (device threads) that fills every SM of the current
   device once for the given medium (0 = mcml, 1 = mcvox), math mode and
   block size (0 = default). */
int mcgb_suggest_streams(int medium, int math, uint32_t block_size, uint32_t *streams);

/* Transport runs.  Validates the configuration and the buffer sizes against
   every offset the configuration names, then launches one kernel on the
   stream.  Returns MCGB_E_INVALID / MCGB_E_SIZE before launching anything if
   a check fails. */
int mcgb_mcml_run(const McgbMcmlConfig *cfg, const McgbBuffers *buf, void *stream);
int mcgb_mcvox_run(const McgbMcvoxConfig *cfg, const McgbBuffers *buf, void *stream);

/* No counterpart in the reference.  Homogeneous-cube radius of every voxel
   for the FAST-math voxelized kernels (McgbBuffers.voxel_radius):
   dev_radius[v] (uint8, the voxels' layout) = the largest k <= max_radius
   such that every voxel within Chebyshev distance k of v lies inside the
   grid and holds v's material.  A packet in voxel v whose sampled free path
   is shorter than k * min(voxel size) takes it in one move instead of
   stopping at each same-material wall and drawing a new path length, as
   the reference does (xopto/mcvox/kernel/mcvox.template.c:760-1038); the
   free path is memoryless, so the interaction points have the same
   distribution.  shape = (nx, ny, nz) on the host; max_radius in
   [1, MCGB_VOXEL_RADIUS_MAX].  Launches only. */
#define MCGB_VOXEL_RADIUS_MAX 64u
int mcgb_voxel_radius(const uint8_t *dev_voxels, const int32_t shape[3], uint8_t *dev_radius,
                      uint32_t max_radius, void *stream);

/* Reads the device counter block (synchronizes the stream) and converts the
   status bits into a return code: MCGB_OK, MCGB_E_TIMEOUT or
   MCGB_E_BAD_INDEX.  host_counters may be NULL. */
int mcgb_check_counters(const uint64_t *dev_counters, void *stream,
                        uint64_t *host_counters);

/* Random numbers.  mcgb_rng_safeprimes writes the first n multipliers a of
   the safe-prime table (a*2^32-1 and a*2^31-1 both prime, scanning down
   from 4294967118).  mcgb_rng_init expands a 64-bit initializer into n
   (x, a) stream seeds exactly as the reference's init_RNG; returns
   MCGB_E_INVALID for an invalid initializer. */
int mcgb_rng_safeprimes(uint32_t *host_a, uint32_t n);
int mcgb_rng_init(uint64_t *host_x, uint32_t *host_a, uint32_t n, uint64_t xinit);
/* n uniform random numbers of one stream into dev_out (one device thread,
   like RngKernel). */
int mcgb_rng_dump(uint64_t x, uint32_t a, uint64_t n, float *dev_out, void *stream);

/* FP32 throughput probe: blocks x threads threads each run 16 independent
   fused multiply-add chains for 8 * iters steps (2 flops each), so one launch
   is blocks * threads * iters * 256 flops.  dev_out (blocks floats) receives
   a value only in a case that does not occur, which keeps the chains live.
   It measures the FP32 peak that the transport kernels are compared with;
   it has no counterpart in the reference. */
int mcgb_fp32_fma_rate(uint32_t blocks, uint32_t threads, uint32_t iters, float *dev_out,
                       void *stream);

/* Fill a device uint64 buffer with a value (ScalarFillMcAccu). */
int mcgb_fill_u64(uint64_t *dev, uint64_t n, uint64_t value, void *stream);

/* Sampling volume of packet traces (replaces Mc.sampling_volume and its
   SamplingVolume kernel, xopto/mcml/mc.py:1040-1217,
   xopto/mcbase/kernel/mcsv.template.c:236-421).  For every packet the path
   through the recorded events is walked voxel by voxel; leaving a voxel
   adds uint32(pl_end * length_in_voxel * multiplier * k + 0.5) to its
   tally, where pl_end is the last float of the packet's last recorded event
   (its optical path length when traced), and uint32(pl_end * k + 0.5) goes
   to dev_total_weight[0].  dev_trace: the event floats (16-byte aligned,
   at least num_packets * max_events * 8 floats); dev_counts: one int32 per
   packet, clipped to max_events; a packet with no events is skipped.
   dev_accu holds the voxel tallies from sv->offset on, flat index
   (z * ny + y) * nx + x.  A packet whose walk exceeds 2^26 voxel crossings
   stops and sets MCGB_STATUS_BAD_INDEX in dev_counters[MCGB_CNT_STATUS]
   (may be NULL).  Deterministic: every tally is an integer sum. */
int mcgb_sampling_volume(const McgbSamplingVolume *sv, const float *dev_trace,
                         uint64_t trace_floats, const int32_t *dev_counts,
                         uint64_t *dev_accu, uint64_t accu_size, uint64_t *dev_total_weight,
                         uint64_t *dev_counters, void *stream);

/* Exact integer sum of tally arrays (the cross-replica reduction):
   dst[i] += src[i] for i < n, host memory. */
int mcgb_reduce_tallies(uint64_t *host_dst, const uint64_t *host_src, uint64_t n);

/* --------------------------------------------------------- batched engine */
/* One simulation of the batched engine: a single layer (finite or
   semi-infinite) between two half-spaces, Henyey-Greenstein phase function,
   normally incident Line source, albedo-weight stepping and a radial
   reflectance detector at the top surface (the batched configuration of
   the benchmark suite; each simulation matches an mcml run of that shape). */
typedef struct McgbBatchSim {
    float mua, mus, g, n;               /* sample layer (1/m, 1/m, -, -)     */
    float n_above, n_below;             /* surrounding half-spaces           */
    float thickness;                    /* m; inf = semi-infinite            */
    float reserved;
    uint64_t num_packets;
} McgbBatchSim;                         /* 40 bytes */

typedef struct McgbBatchConfig {
    uint32_t num_sims;
    uint32_t packets_per_item;          /* work item size, multiple of 32    */
    uint32_t block_size;                /* threads per block (multiple of 32)*/
    uint32_t blocks_per_sm;             /* 0 = as many as fit                */
    uint32_t num_bins;                  /* radial bins per simulation        */
    int32_t math;                       /* MCGB_MATH_*                       */
    float inv_dr;                       /* 1/bin width: bins cover
                                           [0, num_bins/inv_dr); radii beyond
                                           land in the last bin (1/m)        */
    float rmax;                         /* packet termination radius (m)     */
    uint64_t seed;                      /* per-packet stream derivation      */
    double deadline_s;                  /* device wall-clock limit, 0 = 300s */
    uint32_t num_multipliers;           /* entries of dev_multipliers        */
    uint32_t reserved;
} McgbBatchConfig;

/* Bytes of scratch that mcgb_batched_run needs for num_sims simulations
   (work-queue counter, packet prefix sums, per-simulation layer tables). */
int mcgb_batched_work_size(uint32_t num_sims, uint64_t *bytes);

/* Runs every simulation to completion in one persistent launch (plus a
   small preparation kernel).  Warps take work items of packets_per_item
   consecutive packets from a device queue and refill idle lanes packet by
   packet; packet k of simulation s uses the MWC stream derived from
   (seed, s, k), so the tallies do not depend on the scheduling.
   dev_sims [num_sims]; dev_multipliers [num_multipliers] safe-prime
   multipliers; dev_tally [num_sims*num_bins] uint64 radial tallies
   (accumulated: the caller zeroes them); dev_work scratch of
   mcgb_batched_work_size bytes (any contents, caller-owned);
   dev_counters [MCGB_NUM_COUNTERS] (zeroed by the caller).  Launches only
   (no synchronisation), so the call can be captured in a CUDA graph. */
int mcgb_batched_run(const McgbBatchConfig *cfg, const McgbBatchSim *dev_sims,
                     const uint32_t *dev_multipliers, uint64_t *dev_tally,
                     void *dev_work, uint64_t *dev_counters, void *stream);

/* Resident blocks per SM of the batched kernel for a block size. */
int mcgb_batched_occupancy(uint32_t block_size, int math, uint32_t *blocks_per_sm);

/* No counterpart in the reference (it has no batched engine).
   mcgb_batched_run for callers that cannot allocate device memory (code in
   another framework's memory pool or a real-time loop that forbids
   cudaMalloc, or a plugin host that hands over only input and output
   buffers): the scratch lives in a fixed device array inside the library,
   sized for at most MCGB_NOALLOC_MAX_SIMS simulations (about 2.2 MB, held by
   every GPU that loads the library until exit).  Larger batches return
   MCGB_E_SIZE.  The caller still passes every input and output.  The first
   call on a device looks up the array's device address; make that call
   before any stream capture.  All calls share the array: calls that overlap
   on the GPU race and must be serialized by the caller.  No device memory is
   allocated or freed. */
#define MCGB_NOALLOC_MAX_SIMS 8192u
int mcgb_batched_run_noalloc(const McgbBatchConfig *cfg, const McgbBatchSim *dev_sims,
                             const uint32_t *dev_multipliers, uint64_t *dev_tally,
                             uint64_t *dev_counters, void *stream);

/* ------------------------------------------------------ MLP surrogate */
/* Kernels of the radial-reflectance surrogate (a small MLP).  Matrices are
   row-major; bf16 values are passed as uint16_t bit patterns; every GEMM
   accumulates in FP32 on the tensor cores.  Requirements: M % 8 == 0,
   N % 16 == 0, K % 16 == 0 (pad the narrow input and output layers).
   act: 0 = identity, 1 = GELU (tanh form). */

/* Y[M,N] = act(X[M,K] W[N,K]^T + b[N]) stored as bf16; when pre != NULL the
   FP32 pre-activation is stored as well (for the backward pass; for the
   output layer it is the FP32 network output). */
int mcgb_mlp_linear_fwd(const uint16_t *dev_x, const uint16_t *dev_w, const float *dev_b,
                        uint16_t *dev_y, float *dev_pre, int m, int n, int k, int act,
                        void *stream);

/* dPre[M,N] = dY[M,N] * act'(pre) (bf16) and db[N] = sum over rows of dPre
   (FP32, overwritten, summed in a fixed order through dev_scratch of
   mcgb_mlp_act_bwd_scratch(m, n) floats). */
int mcgb_mlp_act_bwd(const uint16_t *dev_dy, const float *dev_pre, uint16_t *dev_dpre,
                     float *dev_db, float *dev_scratch, int m, int n, int act, void *stream);
uint64_t mcgb_mlp_act_bwd_scratch(int m, int n);

/* dX[M,K] = dPre[M,N] W[N,K], with the weight given transposed as
   Wt[K,N] (the optimizer keeps both copies). */
int mcgb_mlp_linear_bwd_input(const uint16_t *dev_dpre, const uint16_t *dev_wt,
                              uint16_t *dev_dx, int m, int n, int k, void *stream);

/* dW[N,K] = dPre[M,N]^T X[M,K] (FP32, overwritten).  The rows are split
   into fixed slices whose partial sums go to dev_scratch and are added in
   a fixed order, so the result is deterministic; dev_scratch holds
   mcgb_mlp_bwd_weight_scratch(m, n, k) floats. */
int mcgb_mlp_linear_bwd_weight(const uint16_t *dev_dpre, const uint16_t *dev_x, float *dev_dw,
                               float *dev_scratch, int m, int n, int k, void *stream);
uint64_t mcgb_mlp_bwd_weight_scratch(int m, int n, int k);

/* Loss gradient of the FP32 network output Y[M,N] (the last layer's
   pre-activation) on the first n_valid of N columns, with optional column
   weights W[N] (NULL = 1); other columns get 0.  Everything is divided by
   M*n_valid; dY is stored as bf16 and the per-block loss partial sums go to
   dev_loss[ceil(M/256)].
     mode 0, squared error:  loss W (Y - T)^2, dY = 2 W (Y - T);
     mode 1, relative error of R = exp(scale*Y) against a target T in the
       same (linear) units:  loss W (T/R - 1)^2, dY = -2 scale W (min(T/R, 4) - 1),
       the gradient with the denominator held at the current R, whose fit
       is the mean of T (unbiased in linear units).  */
int mcgb_mlp_loss_grad(const float *dev_y, const float *dev_t, const float *dev_w,
                       uint16_t *dev_dy, float *dev_loss, int m, int n, int n_valid, int mode,
                       float scale, void *stream);

/* Weight gradient of an input fed as two columns (the high and the low bf16
   part of one FP32 value, so that the FP32-accumulating GEMM sees the input
   at about 16 bits instead of bf16's 8): for j < count, dW[r, j] and
   dW[r, j + shift] both become their sum (rows x cols row-major, FP32).
   AdamW then moves the two copies of each weight alike. */
int mcgb_mlp_tie_columns(float *dev_dw, int rows, int cols, int count, int shift, void *stream);

/* One tensor of a multi-tensor AdamW step (mcgb_mlp_adamw_multi): FP32
   master weights w[rows*cols], their bf16 copy, optionally the transposed
   bf16 copy wt_bf16[cols,rows] (NULL = none), the FP32 gradient, the two
   FP32 moments, and the tensor's decoupled weight decay. */
typedef struct McgbAdamwTensor {
    float *w;
    uint16_t *w_bf16;
    uint16_t *wt_bf16;
    const float *grad;
    float *m;
    float *v;
    int32_t rows, cols;
    float weight_decay;
    int32_t reserved;
} McgbAdamwTensor;                       /* 64 bytes */

#define MCGB_ADAMW_MAX_TENSORS 16

/* mcgb_mlp_adamw on 1..MCGB_ADAMW_MAX_TENSORS tensors in one launch, with
   the same arithmetic per element; `tensors` is a host array, read before
   the call returns. */
int mcgb_mlp_adamw_multi(const McgbAdamwTensor *tensors, int count, float lr, float beta1, float beta2,
                         float eps, int step, void *stream);

/* GEMM implementation behind the mcgb_mlp_* calls: 0 = tcgen05.mma on
   128 x 64 tiles with the FP32 accumulator in tensor memory (the default),
   1 = the warp-level mma.sync kernel on 64 x 64 tiles.  path = -1 only
   queries.  Returns the path in effect before the call, or -1 for an
   invalid path.  Process-wide; do not switch while MLP calls are queued on
   another thread. */
int mcgb_mlp_gemm_path(int path);

/* AdamW on FP32 master weights w[rows*cols] (decoupled weight decay); also
   writes the bf16 copy w_bf16[rows,cols] and, when wt_bf16 != NULL, the
   transposed bf16 copy wt_bf16[cols,rows].  step counts from 1. */
int mcgb_mlp_adamw(float *dev_w, uint16_t *dev_w_bf16, uint16_t *dev_wt_bf16,
                   const float *dev_grad, float *dev_m, float *dev_v, int rows, int cols,
                   float lr, float beta1, float beta2, float eps, float weight_decay, int step,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* XOPTO_GB300_H */
