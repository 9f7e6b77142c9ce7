"""Layered-medium Monte Carlo simulator, a drop-in for xopto.mcml.mc.Mc
(xopto/mcml/mc.py:75-1597) backed by the GB300 transport kernel.

    >>> from pyxopto_gb300.mcml import mc
    >>> layers = mc.mclayer.Layers([
    ...     mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0)),
    ...     mc.mclayer.Layer(d=10e-3, n=1.33, mua=1e2, mus=1e4, pf=mc.mcpf.Hg(0.8)),
    ...     mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0))])
    >>> det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(mc.mcdetector.Axis(0, 5e-3, 50)))
    >>> trace, fluence, detectors = mc.Mc(layers, mc.mcsource.Line(), det).run(1e6)

``cl_devices``, ``cl_build_options`` and ``cl_profiling`` are accepted for
compatibility and ignored: the kernels are prebuilt for sm_103a and run on
the current CUDA device.
"""
import time
from typing import Tuple

import numpy as np

from .. import _abi, _lib
from .._engine import McEngine, torch_cuda
from ..mcbase.mcutil import Axis, RadialAxis
from . import (mclayer, mcsource, mcdetector, mcpf, mcfluence, mctrace, mcoptions, mctypes,
               mcsurface, mcsv)

MC_RESULT_TYPE = Tuple[mctrace.Trace, mcfluence.Fluence, mcdetector.Detectors]


class Mc(McEngine):
    MEDIUM = 0

    def __init__(self, layers, source, detectors=None, trace=None, fluence=None, surface=None,
                 types=mctypes.McDataTypesSingle, options=None, rnginit=None,
                 cl_devices=None, cl_build_options=None, cl_profiling=False):
        super().__init__(options=options, rnginit=rnginit, types=types)
        if surface is not None and not isinstance(surface, mcsurface.SurfaceLayouts):
            raise TypeError('surface must be a SurfaceLayouts instance')
        self._surface = surface
        self._layers = mclayer.Layers(layers)
        self._layers.check()
        self._pf_type = type(self._layers[0].pf)
        self._source = source
        self._source_type = type(source)
        self._detectors = detectors
        self._trace = trace
        self._fluence = fluence

    # ------------------------------------------------------------ properties
    layers = property(lambda self: self._layers)
    source = property(lambda self: self._source)
    detectors = property(lambda self: self._detectors)
    trace = property(lambda self: self._trace)
    fluence = property(lambda self: self._fluence)
    surface = property(lambda self: self._surface)

    def layer(self, index: int) -> mclayer.Layer:
        return self._layers[index]

    def layer_index(self, z: float) -> int:
        """Index of the layer that contains depth z (surrounding media excluded)."""
        top = 0.0
        for i, l in enumerate(self._layers[1:-1], start=1):
            if top <= z < top + l.d:
                return i
            top += l.d
        return 0 if z < 0.0 else len(self._layers) - 1

    # --------------------------------------------------------------- packing
    def pack(self, nphotons: int, num_streams: int = 1) -> _abi.McgbMcmlConfig:
        """Pack every plugin into the C-ABI configuration (the reference's
        _pack, xopto/mcml/mc.py:466-529)."""
        self._clear_allocators()
        if type(self._layers[1].pf) != self._pf_type:
            raise ValueError('The scattering phase function kind/type must not change '
                             'between simulation calls!')
        if type(self._source) != self._source_type:
            raise ValueError('The photon packet source type/kind must not change '
                             'between simulation calls!')
        cfg = _abi.McgbMcmlConfig()
        cfg.num_packets = int(nphotons)
        cfg.num_streams = int(num_streams)
        cfg.pf_kind = self._pf_type.kind
        cfg.num_layers = len(self._layers)
        self._layers.pack(self, cfg.layers)
        self._source.pack(self, cfg.source)
        if self._detectors is not None:
            self._detectors.pack(self, cfg)
        if self._fluence is not None:
            self._fluence.pack(self, cfg.fluence)
        if self._surface is not None:
            self._surface.pack(self, cfg)
        track_opl = self._detectors is not None and self._detectors.tracks_pathlength()
        if self._trace is not None:
            self._trace.pack(self, cfg.trace, int(nphotons))
            track_opl = track_opl or self._trace.plon
        cfg.opt = self._run_options(track_opl)
        return cfg

    # ------------------------------------------------------------------- run
    def run(self, nphotons: int, out=None, wgsize: int = None, maxthreads: int = None,
            copyseeds: bool = False, exportsrc=None, verbose: bool = False) -> MC_RESULT_TYPE:
        """Simulate nphotons packets; returns new (trace, fluence, detectors)
        result objects, or updates the ones passed in ``out``
        (xopto/mcml/mc.py:730-1018).  wgsize sets the threads per block and
        maxthreads the number of random-number streams (device threads)."""
        torch = torch_cuda()
        lib = _lib.load()
        nphotons = int(nphotons)
        if nphotons < 0:
            raise ValueError('The number of photon packets must not be negative!')
        if out is None:
            out = (None, None, None)
        t0 = time.perf_counter()
        if wgsize is not None:
            self._block_size = int(wgsize)
        fn, cfg, buffers = self._prepare(nphotons, maxthreads)
        t1 = time.perf_counter()
        code, counters = self._launch(fn, cfg, buffers, torch)
        t2 = time.perf_counter()
        self._run_report.update(status=counters[_abi.CNT_STATUS],
                                packets_done=counters[_abi.CNT_PACKETS])
        _lib.check(code)
        self._packets_total += nphotons
        results = self._download(nphotons, out)
        t3 = time.perf_counter()
        self._run_report.update(upload=t1 - t0, execution=t2 - t1, download=t3 - t2,
                                threads=counters[_abi.CNT_THREADS], items=nphotons,
                                steps=counters[_abi.CNT_STEPS], status=counters[_abi.CNT_STATUS],
                                packets_done=counters[_abi.CNT_PACKETS])
        if verbose:
            print('McKernel processed {:,d} packets in {:,d} threads ({:,d} steps):\n'
                  '    uploaded in  : {:10.3f} ms\n    executed in  : {:10.3f} ms\n'
                  '    downloaded in: {:10.3f} ms'.format(
                      nphotons, counters[_abi.CNT_THREADS], counters[_abi.CNT_STEPS],
                      (t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3))
        return results

    def _prepare(self, nphotons, maxthreads=None):
        """Packs the configuration, seeds the device streams and allocates
        the device buffers; returns (C-ABI launch function, config, buffers)."""
        torch = torch_cuda()
        lib = _lib.load()
        cfg = self.pack(nphotons)
        device = torch.device('cuda', torch.cuda.current_device())
        dynamic = cfg.opt.scheduling == _abi.SCHED_DYNAMIC
        if dynamic:
            cfg.num_streams = self._ensure_dynamic_streams(torch, device)
        else:
            n_streams = self.suggested_streams(cfg.opt.math) if maxthreads is None \
                else max(1, int(maxthreads))
            self._ensure_streams(torch, n_streams, device)
            cfg.num_streams = n_streams
        buffers = self._device_buffers(torch, device, self._lut_array(), {'_dynamic': dynamic})
        return lib.mcgb_mcml_run, cfg, buffers

    def _download(self, nphotons, out):
        accu = self._dev['accu'].cpu().numpy().view(np.uint64)
        trace_res, fluence_res, detectors_res = out
        if self._trace is not None:
            flt = self._dev['flt'].cpu().numpy()
            ints = self._dev['int'].cpu().numpy()
            off, n = self._flt.find(self._trace)
            ioff, ni = self._int.find(self._trace)
            if trace_res is None:
                trace_res = mctrace.Trace(self._trace)
            trace_res.update_data(self, flt[off:off + n], ints[ioff:ioff + ni], nphotons)
        if self._fluence is not None:
            off, n = self._acc.find(self._fluence)
            if fluence_res is None:
                fluence_res = mcfluence.Fluence(self._fluence)
            fluence_res.update_data(self, [accu[off:off + n]], nphotons)
        if self._detectors is not None:
            if detectors_res is None:
                detectors_res = mcdetector.Detectors(self._detectors)
            for (slot, det), (_, res) in zip(self._detectors.slots(), detectors_res.slots()):
                if isinstance(det, mcdetector.DetectorDefault):
                    continue
                off, n = self._acc.find(det)
                res.update_data(self, [accu[off:off + n]], nphotons)
        return trace_res, fluence_res, detectors_res

    def rng_test(self, n: int, x: int = None, a: int = None) -> np.ndarray:
        """n uniform random numbers of one stream computed on the device
        (Mc.rng_test, xopto/mcml/mc.py:1320-1362)."""
        torch = torch_cuda()
        lib = _lib.load()
        if x is None or a is None:
            xs, as_ = self.host_seeds(1)
            x = int(xs[0]) if x is None else int(x)
            a = int(as_[0]) if a is None else int(a)
        out = torch.empty((int(n),), dtype=torch.float32, device='cuda')
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(lib.mcgb_rng_dump(int(x), int(a), int(n), out.data_ptr(), stream))
        return out.cpu().numpy()

    def __str__(self):
        return 'Mc(layers={}, source={}, detectors={}, trace={}, fluence={})'.format(
            self._layers, self._source, self._detectors, self._trace, self._fluence)

    __repr__ = __str__
