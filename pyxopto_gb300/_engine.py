"""Run machinery shared by the layered and voxelized simulators: buffer
allocators with the reference's method names (xopto/mcbase/mcworker.py
ClWorker / ClWorkerStandardBufferLutMixin / ClWorkerRngMixin), persistent
random-number streams on the device, and the launch / download cycle of
``Mc.run`` (xopto/mcml/mc.py:730-1018).

Device memory and streams come from PyTorch; the compute is the C-ABI
library.  Nothing here runs the simulation on the CPU.
"""
import ctypes as C
import time
from typing import Dict, List, Tuple

import numpy as np

from . import _abi, _lib
from .mcbase import mcoptions
from .rng import Random


class _Pool:
    """Linear allocator of one device buffer (accumulator, float or int)."""

    def __init__(self):
        self.size = 0
        self.items = []        # (owner, offset, count)

    def clear(self):
        self.size = 0
        self.items = []

    def allocate(self, owner, shape) -> int:
        count = int(np.prod(shape)) if len(shape) else 1
        # keep allocations 16-byte aligned for vectorized trace stores
        offset = (self.size + 3) // 4 * 4
        self.items.append((owner, offset, count))
        self.size = offset + count
        return offset

    def find(self, owner) -> Tuple[int, int]:
        for o, off, n in self.items:
            if o is owner:
                return off, n
        raise KeyError(owner)


def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('A CUDA device is required to run the GB300 simulator '
                           '(there is no CPU fallback).')
    return torch


class McEngine:
    """Base class of mcml.Mc and mcvox.Mc."""
    MEDIUM = 0

    def __init__(self, options=None, rnginit=None, types=None):
        from .mcbase import mctypes
        self._types = mctypes.check(types)
        self._mc_options = list(options or [])
        self._rnginit = rnginit
        self._rmax = float('inf')
        self._acc = _Pool()
        self._flt = _Pool()
        self._int = _Pool()
        self._luts: List[np.ndarray] = []
        self._lut_size = 0
        self._dev = {}                # persistent device tensors
        self._num_streams = None
        self._run_report = {'upload': None, 'download': None, 'execution': None,
                            'threads': None, 'items': None, 'steps': None}
        self._block_size = 0
        self._deadline = 0.0
        self._max_steps = 0
        self._shard = (0, 1)
        self._packets_total = 0          # packets simulated so far (dynamic streams)

    # ------------------------------------------------ reference worker API
    def cl_allocate_rw_accumulator_buffer(self, owner, shape) -> int:
        return self._acc.allocate(owner, shape)

    def cl_allocate_rw_float_buffer(self, owner, shape) -> int:
        return self._flt.allocate(owner, shape)

    def cl_allocate_rw_int_buffer(self, owner, shape) -> int:
        return self._int.allocate(owner, shape)

    def append_r_lut(self, data) -> int:
        data = np.asarray(data, dtype=np.float32).ravel()
        offset = self._lut_size
        self._luts.append(data)
        self._lut_size += data.size
        return offset

    def clear_r_luts(self):
        self._luts = []
        self._lut_size = 0

    def _clear_allocators(self):
        self._acc.clear()
        self._flt.clear()
        self._int.clear()
        self.clear_r_luts()

    types = property(lambda self: self._types)
    options = property(lambda self: self._mc_options)
    run_report = property(lambda self: dict(self._run_report), None, None,
                          'Timing of the latest run: upload, execution, download (s), '
                          'threads, items (packets) and steps.')

    def _get_rmax(self):
        return self._rmax

    def _set_rmax(self, v):
        self._rmax = float(v)

    rmax = property(_get_rmax, _set_rmax, None, 'Radius beyond which packets are terminated (m).')

    def _set_deadline(self, seconds):
        self._deadline = max(0.0, float(seconds or 0.0))

    deadline = property(lambda self: self._deadline, _set_deadline, None,
                        'Device wall-clock limit of one run in seconds (0 = 300 s).  A run '
                        'that reaches it stops, keeps its RNG states and raises McgbError '
                        'with code E_TIMEOUT; the device stays usable.')

    def _set_max_steps(self, n):
        self._max_steps = max(0, int(n or 0))

    max_steps_per_packet = property(lambda self: self._max_steps, _set_max_steps, None,
                                    'Terminate a packet after this many steps (0 = no limit).')

    def _set_packets_per_item(self, n):
        n = int(n or 0)
        if not 0 <= n <= 128:
            raise ValueError('packets_per_item must be in [0, 128]')
        self._packets_per_item = n

    packets_per_item = property(lambda self: getattr(self, '_packets_per_item', 0),
                                _set_packets_per_item, None,
                                'Dynamic scheduling: packets a warp takes from the work queue at '
                                'a time (0 = chosen from the packet count and the grid).  The '
                                'tallies do not depend on it.')

    def shard(self, rank: int, world: int):
        """Use slice ``rank`` of a stream table ``world`` times larger than
        one run needs: replicas on different GPUs then simulate disjoint
        streams, and the sum of their integer tallies equals one run with
        world x the streams (for packet counts divisible by the total
        stream count)."""
        if not (0 <= int(rank) < int(world)):
            raise ValueError('rank must be in [0, world)')
        self._shard = (int(rank), int(world))
        self._num_streams = None
        self._dev.pop('rng_x', None)

    def _resolved_options(self) -> Dict:
        return mcoptions.resolve(self._mc_options)

    def _run_options(self, track_opl: bool) -> _abi.McgbRunOptions:
        res = self._resolved_options()
        o = _abi.default_options()
        o.method = int(res.get('MC_METHOD', 0))
        fast = bool(res.get('MC_USE_NATIVE_MATH', False) or res.get('MC_USE_HALF_MATH', False))
        o.math = _abi.MATH_FAST if fast else _abi.MATH_EXACT
        o.use_lottery = int(bool(res.get('MC_USE_LOTTERY', True)))
        o.packet_weight_min = float(res.get('MC_PACKET_WEIGHT_MIN', 1e-4))
        o.lottery_chance = float(res.get('MC_PACKET_LOTTERY_CHANCE', 0.1))
        o.rmax = self._rmax
        o.track_optical_pathlength = int(bool(track_opl))
        o.block_size = self._block_size
        o.deadline_s = self._deadline
        o.max_steps_per_packet = self._max_steps
        if res.get('MCGB_SCHEDULING', 'dynamic') == 'dynamic':
            o.scheduling = _abi.SCHED_DYNAMIC
            if self._rnginit is None:
                self._rnginit = Random().initializer()
            rank, world = self._shard
            o.seed = (int(self._rnginit) + 0x9E3779B97F4A7C15 * rank) & 0xFFFFFFFFFFFFFFFF
            o.packet_offset = self._packets_total
            o.packets_per_item = self.packets_per_item
        else:
            o.scheduling = _abi.SCHED_STATIC
        return o

    DYNAMIC_MULTIPLIERS = 4096

    def dynamic_multipliers(self) -> np.ndarray:
        """Multipliers of the per-packet streams (dynamic scheduling): the
        first entries of the safe-prime table."""
        return Random().multipliers(self.DYNAMIC_MULTIPLIERS)

    def _lut_array(self) -> np.ndarray:
        if not self._luts:
            return np.zeros((0,), dtype=np.float32)
        return np.concatenate(self._luts).astype(np.float32)

    # ------------------------------------------------------------- streams
    def suggested_streams(self, math: int) -> int:
        lib = _lib.load()
        torch_cuda()
        n = C.c_uint32(0)
        _lib.check(lib.mcgb_suggest_streams(self.MEDIUM, int(math), self._block_size, C.byref(n)))
        return int(n.value)

    def host_seeds(self, n: int):
        """(x, a) of the first n streams for this simulator's initializer."""
        if self._rnginit is None:
            self._rnginit = Random().initializer()
        rank, world = self._shard
        if world == 1:
            return Random().seeds(n, self._rnginit)
        x, a = Random().seeds(n * world, self._rnginit)
        return x[rank * n:(rank + 1) * n].copy(), a[rank * n:(rank + 1) * n].copy()

    def _ensure_dynamic_streams(self, torch, device):
        if self._dev.get('dyn_mult') is None:
            a = self.dynamic_multipliers()
            self._dev['dyn_mult'] = torch.from_numpy(a.view(np.int32)).to(device)
            self._dev['dyn_x'] = torch.zeros((1,), dtype=torch.int64, device=device)
        return self.DYNAMIC_MULTIPLIERS

    def _ensure_streams(self, torch, n: int, device):
        """Allocates and seeds n device streams once; their x states persist
        across runs so successive runs continue the streams (the reference
        keeps rng_seeds_x in device memory, xopto/mcml/mc.py:829-845)."""
        if self._num_streams == n and 'rng_x' in self._dev:
            return
        x, a = self.host_seeds(n)
        self._dev['rng_x'] = torch.from_numpy(x.view(np.int64)).to(device)
        self._dev['rng_a'] = torch.from_numpy(a.view(np.int32)).to(device)
        self._num_streams = n

    def rng_states(self) -> np.ndarray:
        """Current x states of the device streams (copyseeds)."""
        if 'rng_x' not in self._dev:
            return None
        return self._dev['rng_x'].cpu().numpy().view(np.uint64).copy()

    # ----------------------------------------------------------- run cycle
    def _device_buffers(self, torch, device, lut: np.ndarray, extra: dict) -> _abi.McgbBuffers:
        d = self._dev
        d['accu'] = torch.zeros((max(self._acc.size, 1),), dtype=torch.int64, device=device)
        d['flt'] = torch.zeros((max(self._flt.size, 4),), dtype=torch.float32, device=device)
        d['int'] = torch.zeros((max(self._int.size, 1),), dtype=torch.int32, device=device)
        d['lut'] = torch.from_numpy(lut if lut.size else np.zeros((1,), np.float32)).to(device)
        d['counters'] = torch.zeros((_abi.NUM_COUNTERS,), dtype=torch.int64, device=device)
        b = _abi.McgbBuffers()
        if 'dyn_mult' in d and extra.pop('_dynamic', False):
            b.rng_x = d['dyn_x'].data_ptr()
            b.rng_a = d['dyn_mult'].data_ptr()
        else:
            b.rng_x = d['rng_x'].data_ptr()
            b.rng_a = d['rng_a'].data_ptr()
        b.accumulator = d['accu'].data_ptr()
        b.accumulator_size = self._acc.size
        b.float_buffer = d['flt'].data_ptr()
        b.float_size = self._flt.size
        b.int_buffer = d['int'].data_ptr()
        b.int_size = self._int.size
        b.fp_lut = d['lut'].data_ptr() if lut.size else None
        b.fp_lut_size = int(lut.size)
        for k, v in extra.items():
            setattr(b, k, v)
        b.counters = d['counters'].data_ptr()
        return b

    def sampling_volume(self, trace, sv, wgsize: int = None, maxthreads: int = None,
                        exportsrc=None, verbose: bool = False):
        """Adds the sampling volume of a trace to ``sv`` and returns it
        (xopto/mcml/mc.py:1040-1217).  Every packet of the trace is walked
        through the voxels of ``sv`` on the GPU; ``wgsize``, ``maxthreads``
        and ``exportsrc`` are accepted for compatibility and ignored."""
        if self._trace is None:
            raise RuntimeError('This Monte Carlo simulator was built without the Trace '
                               'functionality (the trace argument of Mc.__init__ was None)! '
                               'Sampling volume analysis requires trace functionality!')
        torch = torch_cuda()
        lib = _lib.load()
        t0 = time.perf_counter()
        device = torch.device('cuda', torch.cuda.current_device())
        cfg = sv.pack(self)
        nphotons = len(trace)
        cfg.max_events = trace.maxlen
        cfg.num_packets = nphotons
        n_vox = int(np.prod(sv.shape))
        d = self._dev
        if nphotons:
            events = np.ascontiguousarray(trace.data).view(np.float32).reshape(-1)
            d['sv_trace'] = torch.from_numpy(events).pin_memory().to(device, non_blocking=True)
            d['sv_counts'] = torch.from_numpy(np.ascontiguousarray(trace.n, dtype=np.int32)).to(device)
        d['sv_accu'] = torch.zeros((n_vox,), dtype=torch.int64, device=device)
        d['sv_total'] = torch.zeros((1,), dtype=torch.int64, device=device)
        d['counters'] = torch.zeros((_abi.NUM_COUNTERS,), dtype=torch.int64, device=device)
        stream = torch.cuda.current_stream().cuda_stream
        t1 = time.perf_counter()
        if nphotons:
            _lib.check(lib.mcgb_sampling_volume(
                C.byref(cfg), C.c_void_p(d['sv_trace'].data_ptr()), int(d['sv_trace'].numel()),
                C.c_void_p(d['sv_counts'].data_ptr()), C.c_void_p(d['sv_accu'].data_ptr()), n_vox,
                C.c_void_p(d['sv_total'].data_ptr()), C.c_void_p(d['counters'].data_ptr()),
                C.c_void_p(stream)))
        counters = (C.c_uint64 * _abi.NUM_COUNTERS)()
        code = lib.mcgb_check_counters(C.c_void_p(d['counters'].data_ptr()), C.c_void_p(stream),
                                       counters)
        t2 = time.perf_counter()
        _lib.check(code)
        accu = d['sv_accu'].cpu().numpy().view(np.uint64)
        total = d['sv_total'].cpu().numpy().view(np.uint64)
        sv.update_data(self, accumulators=[accu], nphotons=nphotons, total_weight=total)
        t3 = time.perf_counter()
        self._run_report.update(upload=t1 - t0, execution=t2 - t1, download=t3 - t2,
                                items=nphotons, threads=None)
        if verbose:
            print('SamplingVolume processed {:d} packets:\n'
                  '    uploaded/built in: {:10.3f} ms\n'
                  '    executed in      : {:10.3f} ms\n'
                  '    downloaded in    : {:10.3f} ms'.format(
                      nphotons, (t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3))
        return sv

    def _launch(self, lib_fn, cfg, buffers, torch):
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(lib_fn(C.byref(cfg), C.byref(buffers), C.c_void_p(stream)))
        counters = (C.c_uint64 * _abi.NUM_COUNTERS)()
        code = _lib.load().mcgb_check_counters(C.c_void_p(self._dev['counters'].data_ptr()),
                                               C.c_void_p(stream), counters)
        return code, [int(v) for v in counters]
