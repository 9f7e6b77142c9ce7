"""ctypes front-end of the CPU parity oracle (oracle/mcoracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  It runs the restated reference algorithm on
the host for the same packed configuration and seeds as a GPU run, so the
two sets of integer tallies can be compared.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, '_build', 'libmcoracle.so')

LIBM, PORTABLE = 0, 1

_lib = None


def build():
    subprocess.run(['make', '-s', '-C', HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        vp = C.c_void_p
        lib.mco_mcml_run.restype = C.c_uint64
        lib.mco_mcml_run.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_uint64, vp, vp, C.c_int]
        lib.mco_mcvox_run.restype = C.c_uint64
        lib.mco_mcvox_run.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_uint64, vp, vp, C.c_int]
        lib.mco_rng_dump.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, vp]
        lib.mco_pm_log.restype = C.c_float
        lib.mco_pm_log.argtypes = [C.c_float]
        lib.mco_pm_exp.restype = C.c_float
        lib.mco_pm_exp.argtypes = [C.c_float]
        lib.mco_pm_pow.restype = C.c_float
        lib.mco_pm_pow.argtypes = [C.c_float, C.c_float]
        lib.mco_pm_cbrt.restype = C.c_float
        lib.mco_pm_cbrt.argtypes = [C.c_float]
        lib.mco_pm_sincos.argtypes = [C.c_float, vp, vp]
        lib.mco_sizeof.argtypes = [C.c_int]
        lib.mco_sampling_volume.restype = C.c_uint64
        lib.mco_sampling_volume.argtypes = [vp, vp, vp, vp, vp]
        lib.mco_batched_run.restype = C.c_uint64
        lib.mco_batched_run.argtypes = [C.c_int, vp, vp, vp, vp, C.c_int]
        _lib = lib
    return _lib


def run(mc, nphotons: int, streams: int, math: int = LIBM, nthreads: int = 1, seeds=None):
    """Runs a pyxopto_gb300 simulator's packed configuration on the CPU.

    Returns a dict with the raw uint64 accumulator, the per-owner tallies
    ('top', 'bottom', 'specular', 'fluence'), trace buffers, the final RNG
    states and the number of interaction steps."""
    lib = load()
    if mc.MEDIUM == 0:
        cfg = mc.pack(nphotons, streams)
        mats = None
    else:
        cfg, mats = mc.pack(nphotons, streams)
    from pyxopto_gb300 import _abi
    if cfg.opt.scheduling == _abi.SCHED_DYNAMIC:
        a = mc.dynamic_multipliers()
        x = np.zeros((1,), dtype=np.uint64)
        cfg.num_streams = a.size
    elif seeds is None:
        x, a = mc.host_seeds(streams)
    else:
        x, a = seeds
    x = np.ascontiguousarray(x, dtype=np.uint64).copy()
    a = np.ascontiguousarray(a, dtype=np.uint32)
    accu = np.zeros((max(mc._acc.size, 1),), dtype=np.uint64)
    flt = np.zeros((max(mc._flt.size, 1),), dtype=np.float32)
    ints = np.zeros((max(mc._int.size, 1),), dtype=np.int32)
    lut = mc._lut_array()
    lut_p = lut.ctypes.data if lut.size else None
    if mc.MEDIUM == 0:
        steps = lib.mco_mcml_run(int(math), C.addressof(cfg), lut_p, x.ctypes.data, a.ctypes.data,
                                 accu.ctypes.data, accu.size, flt.ctypes.data, ints.ctypes.data,
                                 int(nthreads))
    else:
        vox = np.ascontiguousarray(mc.voxels.data(), dtype=np.uint8).reshape(-1)
        steps = lib.mco_mcvox_run(int(math), C.addressof(cfg), C.addressof(mats), vox.ctypes.data,
                                  lut_p, x.ctypes.data, a.ctypes.data, accu.ctypes.data, accu.size,
                                  flt.ctypes.data, ints.ctypes.data, int(nthreads))
    out = {'accu': accu, 'rng_x': x, 'steps': int(steps), 'float': flt, 'int': ints}
    out.update(tallies(mc, accu))
    return out


def tallies(mc, accu):
    """Split a raw accumulator into named tallies."""
    from pyxopto_gb300.mcbase import mcdetector
    res = {}
    if mc.detectors is not None:
        for slot, det in mc.detectors.slots():
            if isinstance(det, mcdetector.DetectorDefault):
                continue
            off, n = mc._acc.find(det)
            res[slot] = np.array(accu[off:off + n], dtype=np.uint64)
    if mc.fluence is not None:
        off, n = mc._acc.find(mc.fluence)
        res['fluence'] = np.array(accu[off:off + n], dtype=np.uint64)
    return res


def rng_dump(x: int, a: int, n: int) -> np.ndarray:
    out = np.zeros((int(n),), dtype=np.float32)
    load().mco_rng_dump(int(x), int(a), int(n), out.ctypes.data)
    return out


def batched_run(bmc, math: int = PORTABLE, nthreads: int = 1, **shape):
    """CPU restatement of a BatchedMc run: returns (tallies (S, bins), steps)."""
    lib = load()
    cfg = bmc.config(**shape)
    mult = np.ascontiguousarray(bmc.multipliers(cfg.num_multipliers), dtype=np.uint32)
    tally = np.zeros((bmc.num_sims * bmc.raxis.n,), dtype=np.uint64)
    steps = lib.mco_batched_run(int(math), C.addressof(cfg), C.addressof(bmc._sims),
                                mult.ctypes.data, tally.ctypes.data, int(nthreads))
    return tally.reshape(bmc.num_sims, bmc.raxis.n), int(steps)


def sampling_volume(sv_cfg, trace_n, trace_data):
    """The sampling volume of a trace (packets in order) on the CPU; sv_cfg
    is a packed pyxopto_gb300 McgbSamplingVolume whose max_events and
    num_packets describe the trace.  Returns (voxel tallies, total weight,
    status bits)."""
    n = np.ascontiguousarray(trace_n, dtype=np.int32)
    f = np.ascontiguousarray(trace_data, dtype=np.float32).reshape(-1)
    assert n.size == sv_cfg.num_packets
    assert f.size >= sv_cfg.num_packets * sv_cfg.max_events * 8
    accu = np.zeros((int(np.prod(list(sv_cfg.shape))),), dtype=np.uint64)
    total = np.zeros((1,), dtype=np.uint64)
    status = load().mco_sampling_volume(C.addressof(sv_cfg), f.ctypes.data, n.ctypes.data,
                                        accu.ctypes.data, total.ctypes.data)
    return accu, total, int(status)
