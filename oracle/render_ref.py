"""Reference CPU build recipe: renders PyXOpto's own McKernel OpenCL program
for a parity scenario and compiles it for the host CPU into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Run in a container where the PyXOpto sources are
importable (REFERENCE below, override with XOPTO_REFERENCE):

    python oracle/render_ref.py c1_line_hg_radial c2_gk_fluence ...

For each scenario this
  1. builds the reference simulator objects (xopto.mcml.mc.Mc /
     xopto.mcvox.mc.Mc) from tests/golden/scenarios.py, with stub modules for
     the absent pyopencl / numba / matplotlib / shapely packages;
  2. lets the reference pack its structs (Mc._pack) and render its OpenCL
     source (Mc._build_src, xopto/mcml/mc.py:531-626);
  3. writes oracle/_ref/<name>.cpp = oracle/ref_shim.h + the rendered program
     (one line changed: its "typedef char int8_t;" clashes with <cstdint>) +
     a driver that calls McKernel once per RNG stream with that stream's
     packet quota (OpenMP over streams);
  4. writes the packed struct bytes, the LUT and the voxels to
     oracle/_ref/<name>.npz, so the build can later run without the
     reference's Python code (the CPU baseline on another machine);
  5. compiles oracle/_ref/<name>.so with g++ -O2 -ffp-contract=off -fopenmp.

Nothing is copied into the repository: oracle/_ref/ is git-ignored.
"""
import ctypes as C
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_DIR = os.path.join(HERE, '_ref')
# This recipe reads the reference sources where the build container mounts
# them; nothing else in the repository names that path.
REFERENCE = os.environ.get('XOPTO_REFERENCE', '/root/reference')

sys.path.insert(0, os.path.join(REPO, 'tests', 'golden'))
import scenarios  # noqa: E402


def _install_stubs():
    class _Any:
        def __init__(self, *a, **k):
            pass

        def __call__(self, *a, **k):
            return _Any()

        def __getattr__(self, n):
            return _Any()

        def __iter__(self):
            return iter([])

        def __bool__(self):
            return False

    def stub(name):
        m = types.ModuleType(name)

        def ga(n):
            if n[:1].isupper():
                return type(n, (_Any,), {})
            return _Any()
        m.__getattr__ = ga
        sys.modules[name] = m
        return m

    for n in ['pyopencl', 'pyopencl.array', 'pyopencl.tools', 'matplotlib', 'matplotlib.pyplot',
              'matplotlib.widgets', 'matplotlib.colors', 'matplotlib.cm', 'shapely',
              'shapely.geometry', 'shapely.ops', 'shapely.affinity']:
        if n not in sys.modules:
            stub(n)
    if 'numba' not in sys.modules:
        nb = stub('numba')
        nb.jit = lambda *a, **k: (lambda f: f)
        nb.njit = nb.jit
    import scipy.integrate as si
    if not hasattr(si, 'simps'):
        si.simps = si.simpson
    if REFERENCE not in sys.path:
        sys.path.insert(0, REFERENCE)


def reference_mc(name):
    """The reference simulator object for a scenario."""
    _install_stubs()
    s = scenarios.ALL[name]
    if s['medium'] == 'mcml':
        from xopto.mcml import mc
        layers = mc.mclayer.Layers([
            mc.mclayer.Layer(d=l['d'], n=l['n'], mua=l['mua'], mus=l['mus'],
                             pf=scenarios._pf(mc, l['pf'])) for l in s['layers']])
        obj = mc.Mc(layers, scenarios._source(mc.mcsource, s['source']),
                    scenarios._detectors(mc, s.get('detectors')),
                    fluence=scenarios._fluence(mc, s.get('fluence')),
                    surface=scenarios._surface(mc, s.get('surface')),
                    trace=scenarios._trace(mc, s.get('trace')),
                    options=scenarios.options(mc, s), rnginit=s['rnginit'])
    else:
        from xopto.mcvox import mc
        g = s['grid']
        A = mc.mcdetector.Axis
        vox = mc.mcgeometry.Voxels(A(*g['x']), A(*g['y']), A(*g['z']))
        mats = mc.mcmaterial.Materials([
            mc.mcmaterial.Material(n=m['n'], mua=m['mua'], mus=m['mus'],
                                   pf=scenarios._pf(mc, m['pf'])) for m in s['materials']])
        obj = mc.Mc(vox, mats, scenarios._source(mc.mcsource, s['source']),
                    scenarios._detectors(mc, s.get('detectors')),
                    fluence=scenarios._fluence(mc, s.get('fluence')),
                    trace=scenarios._trace(mc, s.get('trace')),
                    options=scenarios.options(mc, s), rnginit=s['rnginit'])
        obj.voxels.material[...] = scenarios.voxel_layout(g, s['layout'])
    if 'rmax' in s:
        obj.rmax = s['rmax']
    return obj


DRIVER_MCML = r'''
/* ---- driver (oracle/render_ref.py): one McKernel call per RNG stream ---- */
extern "C" void ref_run(unsigned long num_packets, unsigned num_streams, float rmax,
                        unsigned long *rng_x, const unsigned *rng_a, unsigned num_layers,
                        const void *layers, const void *source, const void *surface,
                        const void *trace, const void *fluence, const void *detectors,
                        const float *lut, int *ibuf, float *fbuf, unsigned long *accu,
                        int nthreads, unsigned long ibuf_stride, unsigned long fbuf_stride) {
    #pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long t = 0; t < (long)num_streams; ++t) {
        unsigned long q = num_packets / num_streams + ((unsigned long)t < num_packets % num_streams);
        if (!q) continue;
        ref_set_global_id((size_t)t);
        mc_cnt_t done = 0;
        uint32_t nk = 0;
        McKernel((mc_cnt_t)q, &done, &nk, rmax, (uint64_t *)rng_x, (const uint32_t *)rng_a,
                 num_layers, (McLayer const *)layers, (McSource const *)source,
                 (McSurfaceLayouts const *)surface, (McTrace const *)trace,
                 (McFluence const *)fluence, (McDetectors const *)detectors, lut,
                 (mc_int_t *)(ibuf + t * ibuf_stride), fbuf + t * fbuf_stride, (mc_accu_t *)accu);
    }
}
'''

DRIVER_MCVOX = r'''
/* ---- driver (oracle/render_ref.py): one McKernel call per RNG stream ---- */
extern "C" void ref_run(unsigned long num_packets, unsigned num_streams, float rmax,
                        unsigned long *rng_x, const unsigned *rng_a, const void *voxel_cfg,
                        const void *voxels, unsigned num_materials, const void *materials,
                        const void *source, const void *surface, const void *trace,
                        const void *fluence, const void *detectors, const float *lut,
                        int *ibuf, float *fbuf, unsigned long *accu, int nthreads,
                        unsigned long ibuf_stride, unsigned long fbuf_stride) {
    #pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long t = 0; t < (long)num_streams; ++t) {
        unsigned long q = num_packets / num_streams + ((unsigned long)t < num_packets % num_streams);
        if (!q) continue;
        ref_set_global_id((size_t)t);
        mc_cnt_t done = 0;
        uint32_t nk = 0;
        McKernel((mc_cnt_t)q, &done, &nk, rmax, (uint64_t *)rng_x, (const uint32_t *)rng_a,
                 (McVoxelConfig const *)voxel_cfg, (McVoxel const *)voxels,
                 (mc_size_t)num_materials, (McMaterial const *)materials,
                 (McSource const *)source, (McSurfaceLayouts const *)surface,
                 (McTrace const *)trace, (McFluence const *)fluence,
                 (McDetectors const *)detectors, lut, (mc_int_t *)(ibuf + t * ibuf_stride),
                 fbuf + t * fbuf_stride, (mc_accu_t *)accu);
    }
}
'''


DRIVER_SV = r'''
/* ---- driver (oracle/render_ref.py): the reference's SamplingVolume kernel
   over all packets of a trace, as one work-item ---- */
#if MC_USE_SAMPLING_VOLUME
extern "C" void ref_sv(unsigned long num_packets, const void *trace, const void *sv,
                       unsigned long *total_weight, int *ibuf, float *fbuf,
                       unsigned long *accu) {
    ref_set_global_id(0);
    mc_cnt_t done = 0;
    uint32_t nk = 0;
    SamplingVolume((mc_cnt_t)num_packets, &done, &nk, (McTrace const *)trace,
                   (McSamplingVolume const *)sv, (mc_accu_t *)total_weight,
                   (mc_int_t *)ibuf, fbuf, (mc_accu_t *)accu);
}
#endif
'''


def _blob(obj, min_size=8):
    if obj is None:
        return np.zeros((min_size,), dtype=np.uint8)
    b = np.frombuffer(bytes(obj), dtype=np.uint8).copy()
    if b.size < min_size:
        b = np.concatenate([b, np.zeros((min_size - b.size,), dtype=np.uint8)])
    return b


def render(name, nphotons=None):
    """Renders, saves and compiles the reference build of one scenario.
    Returns the path of the compiled library."""
    s = scenarios.ALL[name]
    m = reference_mc(name)
    nphotons = int(nphotons or s['nphotons'])
    m._pack(nphotons)
    m._build_src()
    src = m._cl_src.replace('typedef char int8_t;', '/* int8_t comes from <cstdint> */')
    os.makedirs(REF_DIR, exist_ok=True)
    cpp = os.path.join(REF_DIR, name + '.cpp')
    with open(cpp, 'w') as f:
        f.write('#include "../ref_shim.h"\n')
        f.write(src)
        f.write(DRIVER_MCML if s['medium'] == 'mcml' else DRIVER_MCVOX)
        f.write(DRIVER_SV)
    packed = m._packed
    blobs = {
        'medium': np.array([0 if s['medium'] == 'mcml' else 1]),
        'source': _blob(packed['source']),
        'surface': _blob(packed.get('surface_layouts')),
        'trace': _blob(packed.get('trace')),
        'fluence': _blob(packed.get('fluence')),
        'detectors': _blob(packed.get('detectors')),
        'lut': np.asarray(m.float_r_lut_manager.pack_into(dtype=np.float32), dtype=np.float32)
        if len(m.float_r_lut_manager) else np.zeros((1,), np.float32),
        'accu_size': np.array([max(int(m.cl_rw_accumulator_allocator.size), 1)]),
        'rmax': np.array([m.rmax], dtype=np.float32),
    }
    if s['medium'] == 'mcml':
        blobs['layers'] = _blob(packed['layers'])
        blobs['num_layers'] = np.array([len(m.layers)])
    else:
        blobs['voxel_cfg'] = _blob(packed['voxels'])
        blobs['voxels'] = np.ascontiguousarray(m.voxels.data(m)).view(np.uint8).reshape(-1).copy()
        blobs['materials'] = _blob(packed['materials'])
        blobs['num_materials'] = np.array([len(m.materials)])
    # tally offsets by owner name
    offsets = {}
    alloc = m.cl_rw_accumulator_allocator
    if m.detectors is not None:
        for slot in ('top', 'bottom', 'specular'):
            allocs = alloc.allocations(getattr(m.detectors, slot))
            if allocs:
                offsets[slot] = (allocs[0].offset, allocs[0].size)
    if m.fluence is not None:
        a = alloc.allocations(m.fluence)[0]
        offsets['fluence'] = (a.offset, a.size)
    for k, (o, n) in offsets.items():
        blobs['off_' + k] = np.array([o, n])
    if m.trace is not None:
        # per-stream trace buffers: McKernel numbers the packets of each call
        # from 0, so every stream gets its own slice (remapped in run_ref)
        blobs['trace_maxlen'] = np.array([m.trace.maxlen])
        sv_spec = s.get('sampling_volume')
        if sv_spec:
            # the SamplingVolume kernel's arguments, packed as Mc.sampling_volume
            # does after clearing the buffer allocators (xopto/mcml/mc.py:1096-1114)
            for alloc in (m.cl_rw_accumulator_allocator, m.cl_rw_float_allocator,
                          m.cl_rw_int_allocator):
                alloc.clear()
            sv = scenarios._sampling_volume(m, sv_spec)
            blobs['sv_trace'] = _blob(m.trace.cl_pack(m, nphotons=nphotons))
            blobs['sv'] = _blob(sv.cl_pack(m))
            blobs['sv_size'] = np.array([int(np.prod(sv.shape))])
    np.savez_compressed(os.path.join(REF_DIR, name + '.npz'), **blobs)
    return compile_ref(name)


def compile_ref(name):
    cpp = os.path.join(REF_DIR, name + '.cpp')
    so = os.path.join(REF_DIR, name + '.so')
    cmd = ['g++', '-std=c++17', '-O2', '-ffp-contract=off', '-fno-fast-math', '-fopenmp',
           '-fpermissive', '-w', '-fPIC', '-shared', '-o', so, cpp]
    subprocess.run(cmd, check=True)
    return so


def run_ref(name, nphotons, streams, seeds, nthreads=1):
    """Runs a compiled reference build on (x, a) seeds; returns the raw
    accumulator, the named tallies and the final RNG states."""
    d = dict(np.load(os.path.join(REF_DIR, name + '.npz')))
    lib = C.CDLL(os.path.join(REF_DIR, name + '.so'))
    x = np.ascontiguousarray(seeds[0], dtype=np.uint64).copy()
    a = np.ascontiguousarray(seeds[1], dtype=np.uint32)
    accu = np.zeros((int(d['accu_size'][0]),), dtype=np.uint64)
    maxlen = int(d['trace_maxlen'][0]) if 'trace_maxlen' in d else 0
    qmax = -(-int(nphotons) // int(streams))
    istride, fstride = (qmax, qmax * maxlen * 8) if maxlen else (0, 0)
    fbuf = np.zeros((max(16, int(streams) * fstride),), dtype=np.float32)
    ibuf = np.zeros((max(16, int(streams) * istride),), dtype=np.int32)
    p = lambda k: d[k].ctypes.data
    f = lib.ref_run
    f.restype = None
    rmax = C.c_float(float(d['rmax'][0]))
    if int(d['medium'][0]) == 0:
        f(C.c_ulong(int(nphotons)), C.c_uint(int(streams)), rmax, x.ctypes.data_as(C.c_void_p),
          a.ctypes.data_as(C.c_void_p), C.c_uint(int(d['num_layers'][0])), C.c_void_p(p('layers')),
          C.c_void_p(p('source')), C.c_void_p(p('surface')), C.c_void_p(p('trace')),
          C.c_void_p(p('fluence')), C.c_void_p(p('detectors')), C.c_void_p(p('lut')),
          ibuf.ctypes.data_as(C.c_void_p), fbuf.ctypes.data_as(C.c_void_p),
          accu.ctypes.data_as(C.c_void_p), C.c_int(int(nthreads)), C.c_ulong(istride),
          C.c_ulong(fstride))
    else:
        f(C.c_ulong(int(nphotons)), C.c_uint(int(streams)), rmax, x.ctypes.data_as(C.c_void_p),
          a.ctypes.data_as(C.c_void_p), C.c_void_p(p('voxel_cfg')), C.c_void_p(p('voxels')),
          C.c_uint(int(d['num_materials'][0])), C.c_void_p(p('materials')),
          C.c_void_p(p('source')), C.c_void_p(p('surface')), C.c_void_p(p('trace')),
          C.c_void_p(p('fluence')), C.c_void_p(p('detectors')), C.c_void_p(p('lut')),
          ibuf.ctypes.data_as(C.c_void_p), fbuf.ctypes.data_as(C.c_void_p),
          accu.ctypes.data_as(C.c_void_p), C.c_int(int(nthreads)), C.c_ulong(istride),
          C.c_ulong(fstride))
    out = {'accu': accu, 'rng_x': x}
    if maxlen:
        # stream t's j-th packet is packet t + j * streams
        T, N = int(streams), int(nphotons)
        n_ev = np.zeros((N,), np.int32)
        ev = np.zeros((N, maxlen * 8), np.float32)
        for t in range(T):
            q = N // T + (t < N % T)
            pk = t + T * np.arange(q)
            n_ev[pk] = ibuf[t * istride:t * istride + q]
            ev[pk] = fbuf[t * fstride:t * fstride + q * maxlen * 8].reshape(q, maxlen * 8)
        out['trace_n'] = n_ev
        out['trace_data'] = ev.reshape(-1)
    for k in list(d.keys()):
        if k.startswith('off_'):
            o, n = int(d[k][0]), int(d[k][1])
            out[k[4:]] = accu[o:o + n].copy()
    return out


def run_ref_sv(name, trace_n, trace_data):
    """Runs the reference's own SamplingVolume kernel of a rendered build on
    a trace (packets in order); returns (voxel tallies, total weight)."""
    d = dict(np.load(os.path.join(REF_DIR, name + '.npz')))
    lib = C.CDLL(os.path.join(REF_DIR, name + '.so'))
    n = np.ascontiguousarray(trace_n, dtype=np.int32)
    f = np.ascontiguousarray(trace_data, dtype=np.float32)
    accu = np.zeros((int(d['sv_size'][0]),), dtype=np.uint64)
    total = np.zeros((1,), dtype=np.uint64)
    lib.ref_sv.restype = None
    lib.ref_sv(C.c_ulong(n.size), C.c_void_p(d['sv_trace'].ctypes.data),
               C.c_void_p(d['sv'].ctypes.data), total.ctypes.data_as(C.c_void_p),
               n.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p),
               accu.ctypes.data_as(C.c_void_p))
    return accu, total


if __name__ == '__main__':
    names = sys.argv[1:] or list(scenarios.SCENARIOS)
    for n in names:
        print(n, render(n))
