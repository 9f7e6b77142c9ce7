"""ctypes mirrors of the POD structs in ``include/xopto_gb300.h``.

The layouts must match the C header byte for byte; ``check_layout`` compares
every struct size with ``mcgb_sizeof`` of the loaded library (the role of the
reference's ``sizeof_datatypes`` handshake, xopto/mcml/mc.py:674-728).
"""
import ctypes as C

ACCU_K = 8388607
MAX_LAYERS = 64
MAX_MATERIALS = 256
TRACE_ENTRY_LEN = 8

OK, E_INVALID, E_SIZE, E_CUDA, E_TIMEOUT, E_BAD_INDEX, E_UNSUPPORTED = 0, -1, -2, -3, -4, -5, -6

STATUS_TIMEOUT, STATUS_BAD_INDEX, STATUS_STEP_LIMIT, STATUS_ABORTED = 1, 2, 4, 8
CNT_PACKETS, CNT_STEPS, CNT_STATUS, CNT_THREADS, CNT_ABORT, CNT_QUEUE, NUM_COUNTERS = 0, 1, 2, 3, 4, 5, 8
SCHED_STATIC, SCHED_DYNAMIC = 0, 1

METHOD_ALBEDO_WEIGHT, METHOD_ALBEDO_REJECTION, METHOD_MICROSCOPIC_BEER_LAMBERT = 0, 1, 2
PF_HG, PF_GK, PF_LUT, PF_EXT = 0, 1, 2, 3
PF_EXT_HG2, PF_EXT_MHG, PF_EXT_PC, PF_EXT_MPC, PF_EXT_MGK = 0, 1, 2, 3, 4
PF_EXT_GK2, PF_EXT_HGA, PF_EXT_HGDIR = 5, 6, 7
PF_GK2_FLOATS, PF_HGA_FLOATS = 11, 9
SRC_LINE, SRC_GAUSSIAN_BEAM, SRC_UNIFORM_FIBER_NI, SRC_LAMBERTIAN_FIBER_NI = 0, 1, 2, 3
SRC_UNIFORM_FIBER, SRC_LAMBERTIAN_FIBER, SRC_UNIFORM_BEAM, SRC_ISOTROPIC_POINT = 4, 5, 6, 7
SRC_ISOTROPIC_VOXEL = 8
SRC_UNIFORM_RECTANGULAR, SRC_LAMBERTIAN_RECTANGULAR = 9, 10
SRC_UNIFORM_FIBER_LUT_NI, SRC_UNIFORM_FIBER_LUT, SRC_UNIFORM_RECTANGULAR_LUT = 11, 12, 13
SRC_ISOTROPIC_VOXELS = 14
DET_NONE, DET_TOTAL, DET_RADIAL, DET_RADIAL_PL, DET_TOTAL_PL = 0, 1, 2, 3, 4
DET_CARTESIAN, DET_CARTESIAN_PL, DET_SYMMETRIC_X = 5, 6, 7
DET_LINEAR_ARRAY, DET_SIX_AROUND_ONE, DET_FIBER_ARRAY = 8, 9, 10
DET_LINEAR_ARRAY_PL, DET_SIX_AROUND_ONE_PL, DET_FIBER_ARRAY_PL = 11, 12, 13
DET_FIBER_FLOATS = 13
DET_TOTAL_LUT, DET_TOTAL_LUT_PL, DET_FIBER_LUT_ARRAY = 14, 15, 16
DET_LUT_FIBER_FLOATS = 16
FLUENCE_NONE, FLUENCE_DEPOSITION, FLUENCE_RATE = 0, 1, 2
TRACE_NONE, TRACE_START, TRACE_END, TRACE_ALL = 0, 1, 2, 7
MATH_EXACT, MATH_FAST = 0, 1

f32 = C.c_float
u32 = C.c_uint32
i32 = C.c_int32
u64 = C.c_uint64


class McgbPf(C.Structure):
    _fields_ = [('p', f32 * 5), ('lut_offset', u32), ('lut_size', u32), ('ext_kind', u32)]


class McgbLayer(C.Structure):
    _fields_ = [('thickness', f32), ('top', f32), ('bottom', f32), ('n', f32),
                ('cos_critical_top', f32), ('cos_critical_bottom', f32),
                ('mus', f32), ('mua', f32), ('inv_mut', f32), ('mua_inv_mut', f32),
                ('pf', McgbPf)]


class McgbMaterial(C.Structure):
    _fields_ = [('n', f32), ('mus', f32), ('mua', f32), ('inv_mut', f32),
                ('mua_inv_mut', f32), ('reserved', f32 * 3), ('pf', McgbPf)]


class McgbSource(C.Structure):
    _fields_ = [('kind', i32), ('position', f32 * 3), ('direction', f32 * 3),
                ('direction_reflected', f32 * 3), ('reflectance', f32),
                ('transformation', f32 * 9), ('sigma', f32 * 2), ('clip', f32),
                ('layer_index', i32), ('angular', f32), ('lut_offset', u32), ('lut_size', u32)]


class McgbDetector(C.Structure):
    _fields_ = [('kind', i32), ('direction', f32 * 3), ('position', f32 * 2),
                ('r_min', f32), ('inv_dr', f32), ('cos_min', f32), ('n', u32),
                ('log_scale', i32), ('pl_log_scale', i32), ('offset', u64),
                ('pl_min', f32), ('inv_dpl', f32), ('n_pl', u32), ('table_offset', u32),
                ('y_min', f32), ('inv_dy', f32), ('n_y', u32), ('reserved2', u32)]


class McgbFluence(C.Structure):
    _fields_ = [('kind', i32), ('inv_step', f32 * 3), ('top_left', f32 * 3),
                ('shape', u32 * 3), ('k', i32), ('reserved', u32), ('offset', u64)]


class McgbTrace(C.Structure):
    _fields_ = [('flags', i32), ('max_events', u32), ('event_mask', u32),
                ('reserved', u32), ('data_offset', u64), ('count_offset', u64)]


class McgbSamplingVolume(C.Structure):
    _fields_ = [('top_left', f32 * 3), ('voxel_size', f32 * 3), ('shape', u32 * 3),
                ('multiplier', f32), ('offset', u64), ('k', i32), ('max_events', u32),
                ('num_packets', u64)]


class McgbRunOptions(C.Structure):
    _fields_ = [('method', i32), ('math', i32), ('use_lottery', i32),
                ('packet_weight_min', f32), ('lottery_chance', f32), ('rmax', f32),
                ('track_optical_pathlength', i32), ('block_size', u32),
                ('max_steps_per_packet', u64), ('deadline_s', C.c_double),
                ('scheduling', i32), ('packets_per_item', u32), ('seed', u64),
                ('packet_offset', u64)]


SURFACE_NONE, SURFACE_LAMBERTIAN, SURFACE_LINEAR_ARRAY = 0, 1, 2
SURFACE_SIX_AROUND_ONE, SURFACE_FIBER_ARRAY = 3, 4
SURFACE_FIBER_FLOATS = 17


class McgbSurface(C.Structure):
    _fields_ = [('kind', i32), ('n_fibers', u32), ('table_offset', u32), ('table_size', u32)]


class McgbMcmlConfig(C.Structure):
    _fields_ = [('num_packets', u64), ('num_streams', u32), ('pf_kind', i32),
                ('num_layers', u32), ('reserved', u32), ('opt', McgbRunOptions),
                ('source', McgbSource), ('top', McgbDetector), ('bottom', McgbDetector),
                ('specular', McgbDetector), ('fluence', McgbFluence), ('trace', McgbTrace),
                ('surface_top', McgbSurface), ('surface_bottom', McgbSurface),
                ('layers', McgbLayer * MAX_LAYERS)]


class McgbMcvoxConfig(C.Structure):
    _fields_ = [('num_packets', u64), ('num_streams', u32), ('pf_kind', i32),
                ('num_materials', u32), ('reserved', u32), ('opt', McgbRunOptions),
                ('top_left', f32 * 3), ('bottom_right', f32 * 3), ('voxel_size', f32 * 3),
                ('shape', i32 * 3), ('source', McgbSource), ('top', McgbDetector),
                ('bottom', McgbDetector), ('specular', McgbDetector),
                ('fluence', McgbFluence), ('trace', McgbTrace)]


class McgbBuffers(C.Structure):
    _fields_ = [('rng_x', C.c_void_p), ('rng_a', C.c_void_p),
                ('accumulator', C.c_void_p), ('accumulator_size', u64),
                ('float_buffer', C.c_void_p), ('float_size', u64),
                ('int_buffer', C.c_void_p), ('int_size', u64),
                ('fp_lut', C.c_void_p), ('fp_lut_size', u64),
                ('voxels', C.c_void_p), ('materials', C.c_void_p),
                ('voxel_radius', C.c_void_p), ('counters', C.c_void_p)]


class McgbBatchSim(C.Structure):
    _fields_ = [('mua', f32), ('mus', f32), ('g', f32), ('n', f32),
                ('n_above', f32), ('n_below', f32), ('thickness', f32),
                ('reserved', f32), ('num_packets', u64)]


class McgbBatchConfig(C.Structure):
    _fields_ = [('num_sims', u32), ('packets_per_item', u32), ('block_size', u32),
                ('blocks_per_sm', u32), ('num_bins', u32), ('math', i32),
                ('inv_dr', f32), ('rmax', f32), ('seed', u64), ('deadline_s', C.c_double),
                ('num_multipliers', u32), ('reserved', u32)]


class McgbAdamwTensor(C.Structure):
    _fields_ = [('w', C.c_void_p), ('w_bf16', C.c_void_p), ('wt_bf16', C.c_void_p),
                ('grad', C.c_void_p), ('m', C.c_void_p), ('v', C.c_void_p),
                ('rows', i32), ('cols', i32), ('weight_decay', f32), ('reserved', i32)]


ADAMW_MAX_TENSORS = 16

SIZEOF_KINDS = [McgbLayer, McgbSource, McgbDetector, McgbFluence, McgbTrace,
                McgbMaterial, McgbMcmlConfig, McgbMcvoxConfig, McgbBuffers,
                McgbRunOptions, McgbPf, McgbBatchSim, McgbBatchConfig, McgbSurface,
                McgbSamplingVolume, McgbAdamwTensor]


def check_layout(sizeof_fn):
    """Raise TypeError if a ctypes struct size differs from the library's."""
    for kind, T in enumerate(SIZEOF_KINDS):
        n = sizeof_fn(kind)
        if n != C.sizeof(T):
            raise TypeError('Struct {} is {} bytes in Python but {} bytes in the '
                            'library.'.format(T.__name__, C.sizeof(T), n))


def default_options():
    o = McgbRunOptions()
    o.method = METHOD_ALBEDO_WEIGHT
    o.math = MATH_FAST
    o.use_lottery = 1
    o.packet_weight_min = 1e-4
    o.lottery_chance = 0.1
    o.rmax = float('inf')
    o.track_optical_pathlength = 0
    o.block_size = 0
    o.max_steps_per_packet = 0
    o.deadline_s = 0.0
    o.scheduling = SCHED_STATIC
    o.packets_per_item = 0
    o.seed = 0
    o.packet_offset = 0
    return o
