"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run where the PyXOpto sources are importable (the reference tree that
oracle/render_ref.py reads; override with XOPTO_REFERENCE):

    python tests/golden/make_golden.py

Writes
  golden_<scenario>.npz  for every scenario in scenarios.py: the stream seeds
                         produced by the reference's clrng.Random().seeds,
                         and the tallies plus final RNG states of the
                         reference's own McKernel, rendered by its plugins
                         and compiled for the CPU (oracle/render_ref.py),
                         run with one McKernel call per stream.
  rng_tables.npz         samples of the reference's safe-prime multiplier
                         table and of its seed expansion for several
                         initializers.
  ref_seeds.npz          the reference's clrng.Random().seeds(4096, 1): the
                         stream seeds that drive the reference CPU build in
                         the benchmark's reference arm and in the
                         reference-parity tests (`make_golden.py ref_seeds`).
  cuda_mcml_radial.npz   the CUDA-MCML radial reflectance profile that the
                         reference's validation suite compares against
                         (xopto/mcml/test/reference/cuda_singlelayer_linesource_radial.pkl,
                         test xopto/mcml/test/validate.py:219-345).
  cuda_mcml_fiber.npz    the CUDA-MCML fibre reflectances of the 20 x 20
                         (mua, mus') sweep at 5 source-detector separations
                         (xopto/mcml/test/reference/cuda_singlelayer_uniformfiber.pkl,
                         test xopto/mcml/test/validate.py:348-511), with the
                         geometry of that test.
  cuda_mcml_fiber2.npz   the same for the two-layer sample, sweep on the
                         second layer (cuda_doublelayer_uniformfiber.pkl,
                         test validate.py:692-866).
  uniformfiber_trace.npz the geometry of the trace self-consistency test
                         (validate.py:1059-1226); `make_golden.py trace_check`.
  sfdi_30deg_variable_na.npz  the SFDI amplitudes and phases of the 30 degree
                         incidence test (validate.py:867-1050); written by
                         `make_golden.py sfdi`.
  linear_probe_*.npz     the reflectances of the six- and nine-fibre
                         linear-probe tests (single_layer_*_linear_probe.pkl,
                         validate.py:1227-1758); written by
                         `make_golden.py linear_probe`.
"""
import hashlib
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, os.path.join(REPO, 'oracle')]

import scenarios  # noqa: E402
import render_ref  # noqa: E402


def reference_seeds(n, xinit):
    render_ref._install_stubs()
    from xopto.cl import clrng
    return clrng.Random().seeds(n, xinit=xinit)


def reference_filters(name, trace_n, trace_data):
    """Packet counts and event hashes of the traces kept by the reference's
    own Filter (xopto/mcbase/mctrace.py:216-330) for scenarios.TRACE_FILTERS."""
    m = render_ref.reference_mc(name)
    from xopto.mcbase import mctrace
    out = {}
    for i, spec in enumerate(scenarios.TRACE_FILTERS):
        tr = mctrace.Trace(m.trace)
        tr.data = np.frombuffer(trace_data.tobytes(), dtype=tr.dtype(m)).reshape(trace_n.size, -1)
        tr.n = np.asarray(trace_n, dtype=np.int32)
        filt, dropped = mctrace.Filter(**spec)(tr, update=False)
        out['filter{}_n'.format(i)] = np.asarray(filt.n, dtype=np.int32)
        out['filter{}_sha256'.format(i)] = np.array(
            [hashlib.sha256(np.ascontiguousarray(filt.data).tobytes()).hexdigest()])
        out['filter{}_dropped'.format(i)] = np.array([dropped])
    return out


def make_scenario(name):
    s = scenarios.SCENARIOS[name]
    render_ref.render(name)
    x, a = reference_seeds(s['streams'], s['rnginit'])
    out = render_ref.run_ref(name, s['nphotons'], s['streams'], (x, a))
    data = {'seeds_x': x, 'seeds_a': a, 'rng_x_final': out['rng_x'],
            'nphotons': np.array([s['nphotons']]), 'streams': np.array([s['streams']])}
    for k, v in out.items():
        if k not in ('accu', 'rng_x', 'trace_n', 'trace_data'):
            data['tally_' + k] = v
    if 'trace_n' in out:
        data['trace_n'] = out['trace_n']
        data['trace_sha256'] = np.array([hashlib.sha256(out['trace_data'].tobytes()).hexdigest()])
        data.update(reference_filters(name, out['trace_n'], out['trace_data']))
    if s.get('sampling_volume'):
        sv, total = render_ref.run_ref_sv(name, out['trace_n'], out['trace_data'])
        data['sv_accu'] = sv
        data['sv_total'] = total
    np.savez_compressed(os.path.join(HERE, 'golden_{}.npz'.format(name)), **data)
    print(name, {k: int(v.sum()) for k, v in data.items() if k.startswith('tally_')})


def make_ref_seeds(n=4096, xinit=1):
    x, a = reference_seeds(n, xinit)
    np.savez_compressed(os.path.join(HERE, 'ref_seeds.npz'), x=np.asarray(x, np.uint64),
                        a=np.asarray(a, np.uint32), xinit=np.array([xinit], np.uint64))
    print('ref_seeds', n)


def make_rng_tables():
    render_ref._install_stubs()
    from xopto.cl import clrng
    r = clrng.Random()
    a_table = np.asarray(r._primes[:, 0], dtype=np.uint64)
    idx = np.unique(np.concatenate([np.arange(2000), np.arange(2000, a_table.size, 997),
                                    np.arange(a_table.size - 20, a_table.size)]))
    data = {'primes_index': idx, 'primes_a': a_table[idx], 'primes_count': np.array([a_table.size])}
    for xinit in (1, 12345678901, 0x00000000FFFFFFFE):
        x, a = r.seeds(3000, xinit=xinit)
        data['seeds_x_{}'.format(xinit)] = x
        data['seeds_a_{}'.format(xinit)] = a
    np.savez_compressed(os.path.join(HERE, 'rng_tables.npz'), **data)
    print('rng_tables', idx.size)


def make_cuda_mcml():
    path = os.path.join(render_ref.REFERENCE, 'xopto', 'mcml', 'test', 'reference',
                        'cuda_singlelayer_linesource_radial.pkl')
    with open(path, 'rb') as f:
        d = pickle.load(f)
    layers = d['layers']
    np.savez_compressed(
        os.path.join(HERE, 'cuda_mcml_radial.npz'),
        reflectance=np.asarray(d['reflectance'], dtype=np.float64),
        n=np.array([l['basic']['n'] for l in layers]),
        d=np.array([l['basic']['d'] for l in layers]),
        mua=np.array([l['basic']['mua'] for l in layers]),
        mus=np.array([l['basic']['mus'] for l in layers]),
        g=np.array([l['pf']['pfparams'][0] for l in layers]),
        axis=np.array([d['detector']['axis']['start'], d['detector']['axis']['stop'],
                       d['detector']['axis']['n']]),
        cosmin=np.array([d['detector']['cosmin']]),
        rmax=np.array([d['mc']['rmax']]))
    print('cuda_mcml_radial', len(d['reflectance']))


def make_cuda_fiber(double=False):
    name = 'cuda_doublelayer_uniformfiber.pkl' if double else 'cuda_singlelayer_uniformfiber.pkl'
    path = os.path.join(render_ref.REFERENCE, 'xopto', 'mcml', 'test', 'reference', name)
    with open(path, 'rb') as f:
        d = pickle.load(f)
    layers = d['layers']
    lut = d['lut']
    extra = {}
    if double:
        # validate.py:759-790: layer 1 fixed, the (mua, mus') sweep on layer 2
        extra = dict(fixed_layer=np.array([1]), fixed_mua=np.asarray(lut[0]['mua'], np.float64),
                     fixed_musr=np.asarray(lut[0]['musr'], np.float64), sweep_layer=np.array([2]))
        lut = lut[1]
    np.savez_compressed(
        os.path.join(HERE, 'cuda_mcml_fiber2.npz' if double else 'cuda_mcml_fiber.npz'),
        **extra,
        reflectance=np.asarray(d['reflectance'], dtype=np.float64),
        n=np.array([l['basic']['n'] for l in layers]),
        d=np.array([l['basic']['d'] for l in layers]),
        g=np.array([l['pf']['pfparams'][0] for l in layers]),
        fiber=np.array([d['source']['dcore'], d['source']['dcladding'], d['source']['ncore'],
                        d['source']['na']]),
        axis=np.array([d['detector']['axis']['start'], d['detector']['axis']['stop'],
                       d['detector']['axis']['n']]),
        cosmin=np.array([d['detector']['cosmin']]),
        sds=np.asarray(d['detector']['fibers']['sds'], dtype=np.float64),
        sds_dcore=np.array([d['detector']['fibers']['dcore']]),
        mua=np.asarray(lut['mua'], dtype=np.float64),
        musr=np.asarray(lut['musr'], dtype=np.float64),
        rmax=np.array([d['mc']['rmax']]))
    print(name, np.asarray(d['reflectance']).shape)


PROBE_PICKLES = {
    'hg_six': 'single_layer_hg_lut_six_linear_probe.pkl',
    'hg_nine': 'single_layer_hg_lut_nine_linear_probe.pkl',
    'gk_six': 'single_layer_gk_lut_six_linear_probe.pkl',
}


def make_linear_probe(key):
    """Reflectances of the reference's six- and nine-fibre linear-probe
    validation tests (validate.py:1227-1758) with their geometry.  The
    Gegenbauer sweep (30 x 30 x 20 points) keeps every third absorption and
    scattering value and every sixth gamma to stay small."""
    path = os.path.join(render_ref.REFERENCE, 'xopto', 'mcml', 'test', 'reference', PROBE_PICKLES[key])
    with open(path, 'rb') as f:
        d = pickle.load(f)
    layers, lut = d['layers'], d['lut']
    refl = np.asarray(d['reflectance'], dtype=np.float64)
    mua, musr = np.asarray(lut['mua'], np.float64), np.asarray(lut['musr'], np.float64)
    extra = {}
    if key == 'gk_six':
        ia, im, ig = np.arange(0, mua.size, 3), np.arange(0, musr.size, 3), np.arange(0, lut['gamma'].size, 6)
        refl = refl[np.ix_(ia, im, ig)]
        mua, musr = mua[ia], musr[im]
        gamma = np.asarray(lut['gamma'], np.float64)[ig]
        g = float(d['g'])
        params = np.array([lut['pf_params_lut'][(g, float(v))] for v in gamma], dtype=np.float64)
        extra = dict(g=np.array([g]), gamma=gamma, gk_g=params[:, 0], gk_a=params[:, 1])
    pf = np.array([list(l['pf']['pfparams']) + [0.5] * (2 - len(l['pf']['pfparams'])) for l in layers])
    src, srf, det = d['source'], d['surface'], d['detector']
    fib = lambda f: np.array([f['dcore'], f['dcladding'], f['ncore'], f['na']])
    np.savez_compressed(
        os.path.join(HERE, 'linear_probe_{}.npz'.format(key)), **extra,
        reflectance=refl, mua=mua, musr=musr,
        pf_type=np.array([0 if layers[0]['pf']['type'] == 'Hg' else 1]), pf=pf,
        n=np.array([l['basic']['n'] for l in layers]), d=np.array([l['basic']['d'] for l in layers]),
        source_fiber=fib(src['fiber']), source_position=np.array(src['position'], np.float64),
        surface_fiber=fib(srf['fiber']),
        surface=np.array([srf['n'], srf['spacing'], srf['cutout'][0], srf['cutout'][1], srf['cutoutn'],
                          srf['diameter'], srf['reflectivity']], np.float64),
        detector_fiber=fib(det['fiber']), detector=np.array([det['n'], det['spacing']], np.float64),
        rmax=np.array([d['mc']['rmax']]))
    print('linear_probe', key, refl.shape)


def make_sfdi():
    """Spatial-frequency amplitude and phase of the reference's SFDI test
    (30 degree incidence, SymmetricX detector, 45 detector NAs;
    xopto/mcml/test/validate.py:867-1050) with its geometry."""
    path = os.path.join(render_ref.REFERENCE, 'xopto', 'mcml', 'test', 'reference',
                        'single_layer_sfdi_30deg_incidence_variable_na.pkl')
    with open(path, 'rb') as f:
        d = pickle.load(f)
    layers, ax = d['layers'], d['detector']['axis']
    np.savez_compressed(
        os.path.join(HERE, 'sfdi_30deg_variable_na.npz'),
        n=np.array([l['basic']['n'] for l in layers]), d=np.array([l['basic']['d'] for l in layers]),
        mua=np.array([l['basic']['mua'] for l in layers]), mus=np.array([l['basic']['mus'] for l in layers]),
        g=np.array([l['pf']['pfparams'][0] for l in layers]),
        direction=np.array(d['source']['direction'], dtype=np.float64),
        axis=np.array([ax['center'], ax['range'], ax['n_half'], float(ax['logscale'])]),
        frequencies=np.asarray(d['frequencies'], np.float64), na=np.asarray(d['lut']['na'], np.float64),
        amplitude=np.asarray(d['amplitude'], np.float64), phase=np.asarray(d['phase'], np.float64),
        rmax=np.array([d['mc']['rmax']]))
    print('sfdi', np.asarray(d['amplitude']).shape)


def make_trace_check():
    """Geometry of the reference's trace self-consistency test
    (SingleLayerUniformFiberTrace, xopto/mcml/test/validate.py:1059-1226)."""
    path = os.path.join(render_ref.REFERENCE, 'xopto', 'mcml', 'test', 'reference',
                        'single_layer_uniformfiber_trace.pkl')
    with open(path, 'rb') as f:
        d = pickle.load(f)
    layers, src, det = d['layers'], d['source'], d['detector']
    np.savez_compressed(
        os.path.join(HERE, 'uniformfiber_trace.npz'),
        n=np.array([l['basic']['n'] for l in layers]), d=np.array([l['basic']['d'] for l in layers]),
        g=np.array([l['pf']['pfparams'][0] for l in layers]),
        fiber=np.array([src['dcore'], src['dcladding'], src['ncore'], src['na']]),
        axis=np.array([det['axis']['start'], det['axis']['stop'], det['axis']['n']]),
        cosmin=np.array([det['cosmin']]), maxlen=np.array([d['trace']['maxlen']]),
        mua=np.asarray(d['lut']['mua'], np.float64), musr=np.asarray(d['lut']['musr'], np.float64),
        rmax=np.array([d['mc']['rmax']]))
    print('trace check', d['lut'])


if __name__ == '__main__':
    if sys.argv[1:2] == ['ref_seeds']:
        make_ref_seeds()
        sys.exit(0)
    if sys.argv[1:2] == ['trace_check']:
        make_trace_check()
        sys.exit(0)
    if sys.argv[1:2] == ['sfdi']:
        make_sfdi()
        sys.exit(0)
    if sys.argv[1:2] == ['linear_probe']:
        for k in PROBE_PICKLES:
            make_linear_probe(k)
        sys.exit(0)
    names = sys.argv[1:] or list(scenarios.SCENARIOS)
    for n in names:
        make_scenario(n)
    if not sys.argv[1:]:
        make_rng_tables()
        make_ref_seeds()
        make_cuda_mcml()
        make_cuda_fiber()
        make_cuda_fiber(double=True)
