"""Pins the CPU oracle (and the host-side packing of pyxopto_gb300) to the
reference: for every parity scenario, the oracle run in LIBM math mode on the
reference's seeds reproduces the tallies and final RNG states of the
reference's own McKernel bit-for-bit (tests/golden/golden_<scenario>.npz)."""
import os

import numpy as np
import pytest

import scenarios

GOLD = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.mark.parametrize('name', sorted(scenarios.SCENARIOS))
def test_oracle_matches_reference_build(oracle, lib, name):
    g = np.load(os.path.join(GOLD, 'golden_{}.npz'.format(name)))
    s = scenarios.SCENARIOS[name]
    mc = scenarios.build_mc(name)
    x, a = mc.host_seeds(s['streams'])
    assert np.array_equal(x, g['seeds_x']) and np.array_equal(a, g['seeds_a'])
    out = oracle.run(mc, int(g['nphotons'][0]), int(g['streams'][0]), oracle.LIBM, seeds=(x, a))
    tallies = [k for k in g.files if k.startswith('tally_')]
    assert tallies
    for k in tallies:
        assert np.array_equal(out[k[6:]], g[k]), k
    assert np.array_equal(out['rng_x'], g['rng_x_final'])


@pytest.mark.parametrize('name', ['c2_gk_fluence', 'c3_vox_cylinder'])
def test_oracle_threads_equal_serial(oracle, lib, name):
    s = scenarios.SCENARIOS[name]
    mc = scenarios.build_mc(name)
    a = oracle.run(mc, s['nphotons'], s['streams'], oracle.PORTABLE, nthreads=1)
    b = oracle.run(mc, s['nphotons'], s['streams'], oracle.PORTABLE, nthreads=4)
    assert np.array_equal(a['accu'], b['accu'])
    assert np.array_equal(a['rng_x'], b['rng_x'])


@pytest.mark.parametrize('name', ['c1_line_hg_radial', 'c3_vox_cylinder'])
def test_portable_math_statistically_equal_to_libm(oracle, lib, name):
    """The EXACT-mode math changes individual trajectories but not the
    physics: total tallies of the two math modes agree within 4 sigma."""
    s = scenarios.SCENARIOS[name]
    mc = scenarios.build_mc(name)
    n, t = 4 * s['nphotons'], s['streams']
    a = oracle.run(mc, n, t, oracle.LIBM, nthreads=4)
    from pyxopto_gb300.rng import Random
    b = oracle.run(mc, n, t, oracle.PORTABLE, nthreads=4, seeds=Random().seeds(t, 987654321))
    k = 'top'
    ta, tb = a[k].sum() / 8388607.0 / n, b[k].sum() / 8388607.0 / n
    # binomial-like error of a per-packet weight fraction
    sigma = np.sqrt(max(ta * (1 - ta), 1e-12) / n) * np.sqrt(2.0)
    assert abs(ta - tb) < 4 * sigma + 1e-9


def test_mcml_known_answer_specular(oracle, lib):
    """Specular reflectance of the normal Line source for n 1.0 -> 1.33 is
    ((1.33-1)/(1.33+1))^2 = 0.02006 (the reference's R_specular)."""
    mc = scenarios.build_mc('c1_line_hg_radial')
    out = oracle.run(mc, 200, 8, oracle.PORTABLE)
    spec = out['specular'].sum() / 8388607.0 / 200
    assert abs(spec - ((1.33 - 1) / (1.33 + 1)) ** 2) < 1e-6


TRACE_SCENARIOS = sorted(n for n, s in scenarios.SCENARIOS.items() if s.get('trace'))


def _oracle_trace(oracle, name):
    """(trace object, packed simulator) of the oracle's run of a trace scenario."""
    g = np.load(os.path.join(GOLD, 'golden_{}.npz'.format(name)))
    s = scenarios.SCENARIOS[name]
    mc = scenarios.build_mc(name)
    n = int(g['nphotons'][0])
    out = oracle.run(mc, n, int(g['streams'][0]), oracle.LIBM, seeds=mc.host_seeds(s['streams']))
    off, cnt = mc._flt.find(mc.trace)
    ioff, icnt = mc._int.find(mc.trace)
    tr = type(mc.trace)(mc.trace)
    tr.update_data(mc, out['float'][off:off + cnt], out['int'][ioff:ioff + icnt], n)
    return tr, mc, g


@pytest.mark.parametrize('name', TRACE_SCENARIOS)
def test_oracle_trace_matches_reference_build(oracle, lib, name):
    """Event counts and every event float of the oracle's trace equal the
    reference build's (xopto/mcbase/mctrace.py:541-583)."""
    import hashlib
    tr, _, g = _oracle_trace(oracle, name)
    assert np.array_equal(tr.n, g['trace_n'])
    assert hashlib.sha256(np.ascontiguousarray(tr.data).tobytes()).hexdigest() == str(g['trace_sha256'][0])


@pytest.mark.parametrize('name', TRACE_SCENARIOS)
def test_trace_filter_matches_reference(oracle, lib, name):
    """pyxopto_gb300's Filter keeps the same packets as the reference's
    Filter (xopto/mcbase/mctrace.py:216-330), including the drop count of
    overflowing traces."""
    import hashlib
    from pyxopto_gb300.mcml import mctrace
    tr, _, g = _oracle_trace(oracle, name)
    for i, spec in enumerate(scenarios.TRACE_FILTERS):
        out, dropped = mctrace.Filter(**spec)(tr, update=False)
        assert np.array_equal(out.n, g['filter{}_n'.format(i)]), i
        assert hashlib.sha256(np.ascontiguousarray(out.data).tobytes()).hexdigest() == \
            str(g['filter{}_sha256'.format(i)][0]), i
        assert dropped == int(g['filter{}_dropped'.format(i)][0]), i


@pytest.mark.parametrize('name', TRACE_SCENARIOS)
def test_oracle_sampling_volume_matches_reference_build(oracle, lib, name):
    """The oracle's sampling-volume walk reproduces the reference's own
    SamplingVolume kernel (xopto/mcbase/kernel/mcsv.template.c:236-421)
    bit-for-bit on the same trace."""
    tr, mc, g = _oracle_trace(oracle, name)
    sv = scenarios._sampling_volume(mc, scenarios.SCENARIOS[name]['sampling_volume'])
    cfg = sv.pack(mc)
    cfg.max_events, cfg.num_packets = tr.maxlen, len(tr)
    accu, total, status = oracle.sampling_volume(cfg, tr.n, np.ascontiguousarray(tr.data).view(np.float32))
    assert status == 0
    assert np.array_equal(accu, g['sv_accu'])
    assert np.array_equal(total, g['sv_total'])
    assert np.count_nonzero(accu) > 100
