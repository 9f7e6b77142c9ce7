"""Voxelized-medium Monte Carlo simulator, a drop-in for xopto.mcvox.mc.Mc
(xopto/mcvox/mc.py:91-1632) backed by the GB300 transport kernel.

``cl_devices``, ``cl_build_options`` and ``cl_profiling`` are accepted and
ignored; voxels are uint8 material indices (at most 256 materials).
"""
import ctypes as C
import time

import numpy as np

from .. import _abi, _lib
from .._engine import McEngine, torch_cuda
from ..mcbase.mcmaterial import Material, Materials
from ..mcbase.mcutil import Axis, RadialAxis
from . import (mcgeometry, mcsource, mcdetector, mcpf, mcfluence, mctrace, mcoptions, mctypes,
               mcmaterial, mcsv, mcsurface)


class Mc(McEngine):
    MEDIUM = 1

    def __init__(self, voxels, materials, source, detectors=None, trace=None, fluence=None,
                 surface=None, types=mctypes.McDataTypesSingle, options=None, rnginit=None,
                 cl_devices=None, cl_build_options=None, cl_profiling=False):
        super().__init__(options=options, rnginit=rnginit, types=types)
        mcsurface.check_supported(surface)
        self._surface = surface
        self._voxels = voxels
        self._materials = Materials(materials)
        self._pf_type = type(self._materials[0].pf)
        self._source = source
        self._source_type = type(source)
        self._detectors = detectors
        self._trace = trace
        self._fluence = fluence

    voxels = property(lambda self: self._voxels)
    materials = property(lambda self: self._materials)
    source = property(lambda self: self._source)
    detectors = property(lambda self: self._detectors)
    trace = property(lambda self: self._trace)
    fluence = property(lambda self: self._fluence)

    def material(self, index) -> Material:
        """Material by index or at a position.  For a position the lookup
        uses the voxel index tuple (ix, iy, iz) on the [z, y, x] array, as
        the reference does (xopto/mcvox/mc.py:425-450)."""
        material_index = 0
        if isinstance(index, (int, np.integer)):
            material_index = int(index)
        elif self._voxels.contains(index):
            ind = self._voxels.index(index)
            material_index = int(self._voxels[ind])
        return self._materials[material_index]

    def pack(self, nphotons: int, num_streams: int = 1):
        """Returns (config, material table) in C-ABI form."""
        self._clear_allocators()
        for m in self._materials:
            if type(m.pf) != self._pf_type:
                raise ValueError('The scattering phase function kind/type must not change '
                                 'between simulation calls!')
        if type(self._source) != self._source_type:
            raise ValueError('The photon packet source type/kind must not change '
                             'between simulation calls!')
        data = self._voxels.data()
        if data.size and int(data.max()) >= len(self._materials):
            raise ValueError('Voxel material index {} is outside the material list of length '
                             '{}!'.format(int(data.max()), len(self._materials)))
        cfg = _abi.McgbMcvoxConfig()
        cfg.num_packets = int(nphotons)
        cfg.num_streams = int(num_streams)
        cfg.pf_kind = self._pf_type.kind
        cfg.num_materials = len(self._materials)
        self._voxels.pack_geometry(cfg)
        mats = (_abi.McgbMaterial * len(self._materials))()
        for i, m in enumerate(self._materials):
            m.pack(self, mats[i])
        self._source.pack(self, cfg.source)
        if self._detectors is not None:
            self._detectors.pack(self, cfg)
        if self._fluence is not None:
            self._fluence.pack(self, cfg.fluence)
        track_opl = self._detectors is not None and self._detectors.tracks_pathlength()
        if self._trace is not None:
            self._trace.pack(self, cfg.trace, int(nphotons))
            track_opl = track_opl or self._trace.plon
        cfg.opt = self._run_options(track_opl)
        return cfg, mats

    def run(self, nphotons: int, out=None, wgsize: int = None, maxthreads: int = None,
            copyseeds: bool = False, exportsrc=None, verbose: bool = False):
        """Simulate nphotons packets; returns (trace, fluence, detectors)
        (xopto/mcvox/mc.py:772-1066)."""
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
            print('McKernel processed {:,d} packets in {:,d} threads in {:.3f} ms'.format(
                nphotons, counters[_abi.CNT_THREADS], (t2 - t1) * 1e3))
        return results

    def _prepare(self, nphotons, maxthreads=None):
        """Packs the configuration, seeds the device streams, uploads the
        voxels and materials and allocates the device buffers; returns
        (C-ABI launch function, config, buffers)."""
        torch = torch_cuda()
        lib = _lib.load()
        cfg, mats = self.pack(nphotons)
        device = torch.device('cuda', torch.cuda.current_device())
        dynamic = cfg.opt.scheduling == _abi.SCHED_DYNAMIC
        if dynamic:
            cfg.num_streams = self._ensure_dynamic_streams(torch, device)
        else:
            n_streams = self.suggested_streams(cfg.opt.math) if maxthreads is None \
                else max(1, int(maxthreads))
            self._ensure_streams(torch, n_streams, device)
            cfg.num_streams = n_streams
        vox = np.ascontiguousarray(self._voxels.data(), dtype=np.uint8)
        key = (vox.shape, hash(vox.tobytes()))
        if self._dev.get('vox_key') != key:
            self._dev['vox'] = torch.from_numpy(vox.reshape(-1).copy()).to(device)
            self._dev['vox_key'] = key
            self._dev.pop('vox_radius', None)
        radius = None
        if cfg.opt.math == _abi.MATH_FAST and self._free_flight():
            radius = self._voxel_radius(torch, lib, cfg)
        mat_bytes = np.frombuffer(bytes(mats), dtype=np.uint8).copy()
        self._dev['mats'] = torch.from_numpy(mat_bytes).to(device)
        buffers = self._device_buffers(torch, device, self._lut_array(), {
            'voxels': self._dev['vox'].data_ptr(), 'materials': self._dev['mats'].data_ptr(),
            'voxel_radius': radius, '_dynamic': dynamic})
        return lib.mcgb_mcvox_run, cfg, buffers

    # cap of the homogeneous-cube radius table: beyond about 30 voxels a
    # longer radius saves few wall stops
    VOXEL_RADIUS_CAP = 31

    def _free_flight(self) -> bool:
        return bool(self._resolved_options().get('MCGB_VOXEL_FREE_FLIGHT', True))

    def _voxel_radius(self, torch, lib, cfg):
        """Device address of the homogeneous-cube radius table of the current
        voxels (mcgb_voxel_radius), computed once per voxel grid."""
        if 'vox_radius' not in self._dev:
            rad = torch.empty_like(self._dev['vox'])
            shape = (C.c_int32 * 3)(*[int(v) for v in cfg.shape])
            _lib.check(lib.mcgb_voxel_radius(C.c_void_p(self._dev['vox'].data_ptr()), shape,
                                             C.c_void_p(rad.data_ptr()), self.VOXEL_RADIUS_CAP,
                                             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            # a grid without any homogeneous cube (one voxel thick, or a
            # checkerboard) gains nothing from free flight: leave it off
            self._dev['vox_radius'] = rad if int(rad.max().item()) > 0 else None
        rad = self._dev['vox_radius']
        return rad.data_ptr() if rad is not None else None

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

    def __str__(self):
        return 'Mc(voxels={}, materials={}, source={})'.format(
            self._voxels, self._materials, self._source)

    __repr__ = __str__
