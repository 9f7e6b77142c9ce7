"""Simulator options with the reference's names
(xopto/mcbase/mcoptions.py:119-729).

The reference turns options into #defines of a kernel it compiles at run
time; the GB300 kernels are prebuilt and read the same settings from the
run configuration instead.  Options that only steer OpenCL code generation
(memory spaces, packed structs, fluence cache, soft atomics) are accepted and
have no effect.
"""


class McOption:
    def __init__(self, name: str, value):
        self.cl_options = [(name, value)]

    name = property(lambda self: self.cl_options[0][0])
    value = property(lambda self: self.cl_options[0][1])

    def fetch_cl_options(self, mc=None):
        return list(self.cl_options)

    def __repr__(self):
        return "{}('{}', {})".format(type(self).__name__, self.name, self.value)

    __str__ = __repr__


class McBoolOption(McOption):
    def __init__(self, name, value):
        super().__init__(name, bool(value))


class McIntOption(McOption):
    def __init__(self, name, value):
        super().__init__(name, int(value))


class McFloatOption(McOption):
    def __init__(self, name, value):
        super().__init__(name, float(value))


class McTypeOption(McOption):
    pass


class McMethod(McIntOption):
    """Stepping method: albedo weight (0, default), albedo rejection (1) or
    microscopic Beer-Lambert (2)."""
    albedo_weight = McIntOption('MC_METHOD', 0)
    albedo_rejection = McIntOption('MC_METHOD', 1)
    microscopic_beer_lambert = McIntOption('MC_METHOD', 2)
    aw = albedo_weight
    ar = albedo_rejection
    mbl = microscopic_beer_lambert
    default = albedo_weight

    def __init__(self, value=0):
        if isinstance(value, str):
            value = {'aw': 0, 'albedo_weight': 0, 'ar': 1, 'albedo_rejection': 1,
                     'mbl': 2, 'microscopic_beer_lambert': 2}[value]
        if int(value) not in (0, 1, 2):
            raise ValueError('Unknown Monte Carlo method {}!'.format(value))
        super().__init__('MC_METHOD', value)


class McUseNativeMath(McBoolOption):
    """Use the GPU's special-function units for log, sin, cos, pow, exp,
    division and square root (MCGB_MATH_FAST).  Off by default: the kernels
    then evaluate these functions with the library's portable routines and
    IEEE arithmetic (MCGB_MATH_EXACT), which the CPU oracle reproduces
    bit-for-bit."""
    on = McBoolOption('MC_USE_NATIVE_MATH', True)
    off = McBoolOption('MC_USE_NATIVE_MATH', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_NATIVE_MATH', value)


class McScheduling(McOption):
    """How packets are distributed over the GPU threads.

    'dynamic' (default): persistent warps take packets from a device queue
    and refill idle lanes packet by packet; packet p simulates on its own
    multiply-with-carry stream derived from (rnginit, p), so results are
    bit-reproducible and every lane stays busy until the last packets.
    'static': thread t owns stream t of the seed table and simulates packets
    t, t+T, t+2T, ... (the reference's per-thread streams, continued from run
    to run)."""
    static = None
    dynamic = None

    def __init__(self, value: str = 'dynamic'):
        if value not in ('static', 'dynamic'):
            raise ValueError('scheduling must be "static" or "dynamic"')
        super().__init__('MCGB_SCHEDULING', value)


McScheduling.static = McScheduling('static')
McScheduling.dynamic = McScheduling('dynamic')
McScheduling.default = McScheduling.dynamic


class McVoxelFreeFlight(McBoolOption):
    """Voxelized media with native math only (albedo weight and albedo
    rejection, no trace): a packet whose sampled free path stays inside a
    cube of voxels of its own material takes the whole path in one move
    instead of stopping at every voxel wall and drawing a new path there, as
    the reference does.  The free path is memoryless, so the interactions
    have the same distribution; the tallies agree with the reference within
    the Monte Carlo error.  On by default; off restores the wall-by-wall
    walk."""
    on = McBoolOption('MCGB_VOXEL_FREE_FLIGHT', True)
    off = McBoolOption('MCGB_VOXEL_FREE_FLIGHT', False)

    def __init__(self, value: bool = True):
        super().__init__('MCGB_VOXEL_FREE_FLIGHT', value)


McVoxelFreeFlight.default = McVoxelFreeFlight.on


class McUseHalfMath(McBoolOption):
    """Mapped to McUseNativeMath: the GB300 fast path is the narrowest
    precision offered."""
    on = McBoolOption('MC_USE_HALF_MATH', True)
    off = McBoolOption('MC_USE_HALF_MATH', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_HALF_MATH', value)


class McUseLottery(McBoolOption):
    on = McBoolOption('MC_USE_LOTTERY', True)
    off = McBoolOption('MC_USE_LOTTERY', False)
    default = on

    def __init__(self, value: bool = True):
        super().__init__('MC_USE_LOTTERY', value)


class McMinimumPacketWeight(McFloatOption):
    default = McFloatOption('MC_PACKET_WEIGHT_MIN', 1e-4)

    def __init__(self, value: float = 1e-4):
        if 0.0 >= value or value > 1.0:
            raise ValueError('Minimum photon packet weight must be > 0.0 and <= 1.0, '
                             'but got {}!'.format(value))
        super().__init__('MC_PACKET_WEIGHT_MIN', value)


class McPacketLotteryChance(McFloatOption):
    default = McFloatOption('MC_PACKET_LOTTERY_CHANCE', 0.1)

    def __init__(self, value: float = 0.1):
        if 0.0 >= value or value > 1.0:
            raise ValueError('Lottery chance must be > 0.0 and <= 1.0, but got {}!'.format(value))
        super().__init__('MC_PACKET_LOTTERY_CHANCE', value)


class McDebugMode(McBoolOption):
    on = McBoolOption('MC_ENABLE_DEBUG', True)
    off = McBoolOption('MC_ENABLE_DEBUG', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_ENABLE_DEBUG', value)


class McUseFluenceCache(McBoolOption):
    on = McBoolOption('MC_USE_FLUENCE_CACHE', True)
    off = McBoolOption('MC_USE_FLUENCE_CACHE', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_FLUENCE_CACHE', value)


class McUseEvents(McBoolOption):
    """Packet event tracking (xopto/mcbase/mcoptions.py:709-732).  The GPU
    kernels always track events where a trace event mask needs them, so the
    option is accepted and changes nothing; like the reference's constructor
    (which names MC_USE_PACKED_STRUCTURES there), it is only recorded."""
    on = McBoolOption('MC_USE_EVENTS', True)
    off = McBoolOption('MC_USE_EVENTS', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_EVENTS', value)


class McUseSoft64Atomics(McBoolOption):
    on = McBoolOption('MC_USE_SOFT_64_ATOMICS', True)
    off = McBoolOption('MC_USE_SOFT_64_ATOMICS', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_SOFT_64_ATOMICS', value)


class McUsePackedStructures(McBoolOption):
    on = McBoolOption('MC_USE_PACKED_STRUCTS', True)
    off = McBoolOption('MC_USE_PACKED_STRUCTS', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_PACKED_STRUCTS', value)


class McUseEnhancedRng(McBoolOption):
    """Not supported by the GB300 kernels (raises at run)."""
    on = McBoolOption('MC_USE_ENHANCED_RNG', True)
    off = McBoolOption('MC_USE_ENHANCED_RNG', False)
    default = off

    def __init__(self, value: bool = False):
        super().__init__('MC_USE_ENHANCED_RNG', value)


class McFloatLutMemory(McTypeOption):
    global_mem = McTypeOption('MC_FLOAT_LUT_ARRAY_MEMORY', '__global')
    constant_mem = McTypeOption('MC_FLOAT_LUT_ARRAY_MEMORY', '__constant')
    default = constant_mem


class McIntLutMemory(McTypeOption):
    global_mem = McTypeOption('MC_INT_LUT_ARRAY_MEMORY', '__global')
    constant_mem = McTypeOption('MC_INT_LUT_ARRAY_MEMORY', '__constant')
    default = constant_mem


_IGNORED = {'MC_USE_FLUENCE_CACHE', 'MC_USE_SOFT_64_ATOMICS', 'MC_USE_PACKED_STRUCTS',
            'MC_FLOAT_LUT_ARRAY_MEMORY', 'MC_INT_LUT_ARRAY_MEMORY', 'MC_ENABLE_DEBUG',
            'MC_FP_LUT_ARRAY_MEMORY', 'MC_USE_EVENTS'}


def resolve(options) -> dict:
    """Collapse a list of McOption objects or (name, value) tuples into a
    dict; later entries override earlier ones."""
    out = {}
    for item in options or []:
        if isinstance(item, McOption):
            pairs = item.fetch_cl_options()
        elif isinstance(item, (tuple, list)) and len(item) == 2:
            pairs = [tuple(item)]
        else:
            raise ValueError('Simulator options must be a list of McOption or (name, value) tuples!')
        for name, value in pairs:
            out[name] = value
    if out.get('MC_USE_ENHANCED_RNG'):
        raise ValueError('MC_USE_ENHANCED_RNG is not supported by the GB300 kernels.')
    if out.get('MC_USE_DOUBLE_PRECISION'):
        raise ValueError('Double precision is not supported by the GB300 kernels.')
    return out
