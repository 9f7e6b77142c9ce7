"""Loader of the in-tree C-ABI library ``libxopto_gb300.so``.

There is no fallback: if the library is missing the import of a simulator
fails with an explicit error telling the user to build it.
"""
import ctypes as C
import os
import threading

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libxopto_gb300.so')

_lock = threading.Lock()
_lib = None

_vp = C.c_void_p
_SIGNATURES = {
    'mcgb_last_error': (C.c_char_p, []),
    'mcgb_abi_version': (C.c_int, []),
    'mcgb_sizeof': (C.c_int, [C.c_int]),
    'mcgb_suggest_streams': (C.c_int, [C.c_int, C.c_int, C.c_uint32, C.POINTER(C.c_uint32)]),
    'mcgb_mcml_run': (C.c_int, [C.POINTER(_abi.McgbMcmlConfig), C.POINTER(_abi.McgbBuffers), _vp]),
    'mcgb_mcvox_run': (C.c_int, [C.POINTER(_abi.McgbMcvoxConfig), C.POINTER(_abi.McgbBuffers), _vp]),
    'mcgb_check_counters': (C.c_int, [_vp, _vp, C.POINTER(C.c_uint64)]),
    'mcgb_rng_safeprimes': (C.c_int, [_vp, C.c_uint32]),
    'mcgb_rng_init': (C.c_int, [_vp, _vp, C.c_uint32, C.c_uint64]),
    'mcgb_rng_dump': (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint64, _vp, _vp]),
    'mcgb_fill_u64': (C.c_int, [_vp, C.c_uint64, C.c_uint64, _vp]),
    'mcgb_fp32_fma_rate': (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, _vp, _vp]),
    'mcgb_reduce_tallies': (C.c_int, [_vp, _vp, C.c_uint64]),
    'mcgb_sampling_volume': (C.c_int, [C.POINTER(_abi.McgbSamplingVolume), _vp, C.c_uint64, _vp,
                                       _vp, C.c_uint64, _vp, _vp, _vp]),
    'mcgb_voxel_radius': (C.c_int, [_vp, C.POINTER(C.c_int32), _vp, C.c_uint32, _vp]),
}
_OPTIONAL = {
    'mcgb_batched_run': (C.c_int, [C.POINTER(_abi.McgbBatchConfig), _vp, _vp, _vp, _vp, _vp, _vp]),
    'mcgb_batched_occupancy': (C.c_int, [C.c_uint32, C.c_int, C.POINTER(C.c_uint32)]),
    'mcgb_batched_work_size': (C.c_int, [C.c_uint32, C.POINTER(C.c_uint64)]),
    'mcgb_batched_run_noalloc': (C.c_int, [C.POINTER(_abi.McgbBatchConfig), _vp, _vp, _vp, _vp, _vp]),
    'mcgb_mlp_linear_fwd': (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    'mcgb_mlp_act_bwd': (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    'mcgb_mlp_act_bwd_scratch': (C.c_uint64, [C.c_int, C.c_int]),
    'mcgb_mlp_linear_bwd_input': (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    'mcgb_mlp_linear_bwd_weight': (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp]),
    'mcgb_mlp_bwd_weight_scratch': (C.c_uint64, [C.c_int, C.c_int, C.c_int]),
    'mcgb_mlp_tie_columns': (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
    'mcgb_mlp_gemm_path': (C.c_int, [C.c_int]),
    'mcgb_mlp_adamw_multi': (C.c_int, [_vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                       _vp]),
    'mcgb_mlp_loss_grad': (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.c_float, _vp]),
    'mcgb_mlp_adamw': (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_float,
                                 C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _vp]),
}


class McgbError(RuntimeError):
    def __init__(self, code, message):
        super().__init__('{} (code {})'.format(message, code))
        self.code = code


def load():
    """Load the library (once) and check the ABI struct layouts."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                'libxopto_gb300.so is not built ({}). Build it with '
                '"python -m pyxopto_gb300.build" (needs nvcc).'.format(LIB_PATH))
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        for name, (res, args) in _OPTIONAL.items():
            f = getattr(lib, name, None)
            if f is not None:
                f.restype, f.argtypes = res, args
        _abi.check_layout(lib.mcgb_sizeof)
        _lib = lib
        return lib


def check(code: int):
    """Raise McgbError for a negative library return code."""
    if code != 0:
        msg = load().mcgb_last_error().decode(errors='replace')
        raise McgbError(code, msg or 'libxopto_gb300 error')
    return code
