"""Batched Monte Carlo: thousands of independent single-layer simulations,
each with its own optical properties and packet count, in one persistent
work-stealing launch.

The reference runs such sweeps as a sequential loop of ``Mc.run`` calls
(xopto/mcml/mcrun/helper.py:640-686, xopto/mcml/test/validate.py:431-440),
one kernel launch, upload and download per simulation.  ``BatchedMc`` runs
the whole sweep in one launch (``mcgb_batched_run``), optionally replayed
from a captured CUDA graph, with the launch shape chosen by ``autotune``.

    >>> sims = BatchedMc.sample_sims(4096, seed=1)        # the benchmark ranges
    >>> bmc = BatchedMc(sims, raxis=Axis(0.0, 3e-3, 30))
    >>> reflectance = bmc.run()                            # (4096, 30)
"""
import ctypes as C
import json
import os
import time

import numpy as np

from . import _abi, _lib
from .mcbase.mcutil import Axis, RadialAxis
from .rng import Random

_CACHE = os.path.join(os.path.expanduser('~'), '.cache', 'pyxopto_gb300', 'autotune.json')


class BatchedMc:
    """Batch of single-layer simulations: a layer (mua, mus, g, n, thickness)
    between half-spaces n_above / n_below, Henyey-Greenstein phase function,
    normally incident Line source, radial reflectance detector ``raxis``
    (radii beyond the axis go into the last bin, as in Radial)."""

    FIELDS = ('mua', 'mus', 'g', 'n', 'n_above', 'n_below', 'thickness', 'num_packets')

    def __init__(self, sims, raxis: Axis = None, fast: bool = True, seed: int = 1,
                 rmax: float = float('inf'), block_size: int = None, packets_per_item: int = None,
                 blocks_per_sm: int = 0):
        self._raxis = raxis if raxis is not None else Axis(0.0, 3e-3, 30)
        if self._raxis.logscale or self._raxis.start != 0.0:
            raise ValueError('The batched radial detector needs a linear axis starting at 0.')
        self._fast = bool(fast)
        self._seed = int(seed)
        self._rmax = float(rmax)
        self.set_sims(sims)
        self._block_size = block_size
        self._packets_per_item = packets_per_item
        self._blocks_per_sm = int(blocks_per_sm)
        self._dev = {}
        self._graph = None
        self._graph_key = None
        self._last = {}

    # ----------------------------------------------------------- inputs
    @staticmethod
    def sample_sims(num: int, seed: int = 1, packets=(1e4, 1e6)):
        """Draws the benchmark batch: mua ~ logU[1, 1000] 1/m, reduced
        scattering mus' ~ logU[500, 5000] 1/m, g ~ U[0.6, 0.95],
        mus = mus'/(1 - g), n ~ U[1.33, 1.5], semi-infinite layer in air,
        packets ~ round(logU[packets])."""
        rng = np.random.default_rng(seed)
        mua = np.exp(rng.uniform(np.log(1.0), np.log(1000.0), num))
        musr = np.exp(rng.uniform(np.log(500.0), np.log(5000.0), num))
        g = rng.uniform(0.6, 0.95, num)
        n = rng.uniform(1.33, 1.5, num)
        nph = np.round(np.exp(rng.uniform(np.log(packets[0]), np.log(packets[1]), num)))
        return {'mua': mua, 'mus': musr / (1.0 - g), 'g': g, 'n': n,
                'n_above': np.ones(num), 'n_below': np.ones(num),
                'thickness': np.full(num, np.inf), 'num_packets': nph.astype(np.uint64)}

    def set_sims(self, sims):
        """Replace the simulation parameters (dict of arrays or a structured
        array with the FIELDS)."""
        n = len(sims['mua'])
        arr = (_abi.McgbBatchSim * n)()
        a = np.frombuffer(arr, dtype=np.dtype([('mua', 'f4'), ('mus', 'f4'), ('g', 'f4'),
                                                ('n', 'f4'), ('n_above', 'f4'), ('n_below', 'f4'),
                                                ('thickness', 'f4'), ('reserved', 'f4'),
                                                ('num_packets', 'u8')]))
        for f in self.FIELDS:
            if f in ('n_above', 'n_below'):
                a[f] = np.asarray(sims.get(f, np.ones(n)), dtype=np.float32)
            elif f == 'thickness':
                a[f] = np.asarray(sims.get(f, np.full(n, np.inf)), dtype=np.float32)
            else:
                a[f] = np.asarray(sims[f])
        if np.any(a['num_packets'] < 0) or np.any(a['mua'] < 0) or np.any(a['mus'] < 0):
            raise ValueError('negative optical properties or packet counts')
        self._sims = arr
        self._sims_np = a
        self._num = n

    num_sims = property(lambda self: self._num)
    packets = property(lambda self: self._sims_np['num_packets'].astype(np.int64))
    raxis = property(lambda self: self._raxis)
    last_report = property(lambda self: dict(self._last))

    def config(self, block_size=None, packets_per_item=None, blocks_per_sm=None):
        c = _abi.McgbBatchConfig()
        c.num_sims = self._num
        c.packets_per_item = int(packets_per_item or self._packets_per_item or 256)
        c.block_size = int(block_size or self._block_size or 128)
        c.blocks_per_sm = int(self._blocks_per_sm if blocks_per_sm is None else blocks_per_sm)
        c.num_bins = self._raxis.n
        c.math = _abi.MATH_FAST if self._fast else _abi.MATH_EXACT
        c.inv_dr = 1.0 / self._raxis.step
        c.rmax = self._rmax
        c.seed = self._seed
        c.deadline_s = 0.0
        c.num_multipliers = 4096
        return c

    def multipliers(self, n=4096):
        return Random().multipliers(n)

    # --------------------------------------------------------- device run
    def _buffers(self, torch):
        d = self._dev
        lib = _lib.load()
        if d.get('num') != self._num:
            nbytes = C.c_uint64(0)
            _lib.check(lib.mcgb_batched_work_size(self._num, C.byref(nbytes)))
            d['work'] = torch.empty((int(nbytes.value) // 8 + 2,), dtype=torch.int64, device='cuda')
            d['tally'] = torch.zeros((self._num * self._raxis.n,), dtype=torch.int64, device='cuda')
            d['counters'] = torch.zeros((_abi.NUM_COUNTERS,), dtype=torch.int64, device='cuda')
            d['sims'] = torch.empty((C.sizeof(self._sims),), dtype=torch.uint8, device='cuda')
            d['num'] = self._num
        if 'mult' not in d:
            d['mult'] = torch.from_numpy(self.multipliers().view(np.int32)).cuda()
        host = torch.from_numpy(np.frombuffer(self._sims, dtype=np.uint8).copy())
        d['sims'].copy_(host, non_blocking=False)
        return d

    def _launch(self, torch, cfg, d, stream):
        lib = _lib.load()
        d['tally'].zero_()
        d['counters'].zero_()
        _lib.check(lib.mcgb_batched_run(C.byref(cfg), C.c_void_p(d['sims'].data_ptr()),
                                        C.c_void_p(d['mult'].data_ptr()),
                                        C.c_void_p(d['tally'].data_ptr()),
                                        C.c_void_p(d['work'].data_ptr()),
                                        C.c_void_p(d['counters'].data_ptr()),
                                        C.c_void_p(stream)))

    def run_raw(self, graph: bool = False, **shape):
        """Runs the batch; returns the raw uint64 tallies (num_sims, bins).
        With graph=True the zeroing and the launch are captured once into a
        CUDA graph and replayed on later calls with the same shape."""
        import torch
        cfg = self.config(**shape)
        d = self._buffers(torch)
        t0 = time.perf_counter()
        if graph:
            key = (self._num, cfg.packets_per_item, cfg.block_size, cfg.blocks_per_sm, cfg.math,
                   cfg.seed)
            if self._graph is None or self._graph_key != key:
                s = torch.cuda.Stream()
                s.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(s):                  # warm-up outside capture
                    self._launch(torch, cfg, d, s.cuda_stream)
                torch.cuda.current_stream().wait_stream(s)
                torch.cuda.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch(torch, cfg, d, torch.cuda.current_stream().cuda_stream)
                self._graph, self._graph_key = g, key
            self._graph.replay()
        else:
            self._launch(torch, cfg, d, torch.cuda.current_stream().cuda_stream)
        counters = (C.c_uint64 * _abi.NUM_COUNTERS)()
        code = _lib.load().mcgb_check_counters(C.c_void_p(d['counters'].data_ptr()),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                               counters)
        dt = time.perf_counter() - t0
        _lib.check(code)
        self._last = {'seconds': dt, 'steps': int(counters[_abi.CNT_STEPS]),
                      'packets': int(counters[_abi.CNT_PACKETS]), 'graph': bool(graph)}
        return d['tally'].cpu().numpy().view(np.uint64).reshape(self._num, self._raxis.n).copy()

    def run(self, graph: bool = False, **shape) -> np.ndarray:
        """Radial reflectance per simulation (num_sims, bins), normalized as
        Radial.reflectance: raw/K per ring area per packet."""
        raw = self.run_raw(graph=graph, **shape)
        return self.normalize(raw)

    def normalize(self, raw):
        e = self._raxis.edges
        inv_area = 1.0 / (np.pi * (e[1:] ** 2 - e[:-1] ** 2))
        n = np.maximum(self.packets, 1).astype(np.float64)
        return raw.astype(np.float64) / _abi.ACCU_K * inv_area[None, :] / n[:, None]

    # ------------------------------------------------------------ autotune
    def autotune(self, block_sizes=(64, 128, 256), items=(64, 256, 1024), calib_fraction=0.05,
                 cache: str = _CACHE, force: bool = False):
        """Times every (block size, packets per item) pair on a calibration
        subset of the batch (the first ``calib_fraction`` of the packets of
        every simulation) and keeps the fastest; the choice is cached per
        device and math mode in ``cache``."""
        import torch
        dev = torch.cuda.get_device_name()
        key = '{}|{}|bins{}'.format(dev, 'fast' if self._fast else 'exact', self._raxis.n)
        table = {}
        if cache and os.path.exists(cache):
            try:
                with open(cache) as f:
                    table = json.load(f)
            except Exception:
                table = {}
        if key in table and not force:
            best = table[key]
            self._block_size, self._packets_per_item = best['block_size'], best['packets_per_item']
            return best
        saved = self._sims_np['num_packets'].copy()
        self._sims_np['num_packets'] = np.maximum(
            (saved * calib_fraction).astype(np.uint64), 1).astype(np.uint64)
        results = []
        try:
            for bs in block_sizes:
                for it in items:
                    self.run_raw(block_size=bs, packets_per_item=it)          # warm-up
                    ts = []
                    for _ in range(2):
                        self.run_raw(block_size=bs, packets_per_item=it)
                        ts.append(self._last['seconds'])
                    results.append((min(ts), bs, it))
        finally:
            self._sims_np['num_packets'] = saved
        t, bs, it = min(results)
        best = {'block_size': bs, 'packets_per_item': it, 'seconds': t,
                'candidates': [{'seconds': r[0], 'block_size': r[1], 'packets_per_item': r[2]}
                               for r in results]}
        self._block_size, self._packets_per_item = bs, it
        if cache:
            try:
                os.makedirs(os.path.dirname(cache), exist_ok=True)
                table[key] = best
                with open(cache, 'w') as f:
                    json.dump(table, f, indent=1)
            except OSError:
                pass
        return best
