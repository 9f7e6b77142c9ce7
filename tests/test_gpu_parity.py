"""GPU parity: the CUDA kernels against the CPU oracle, through the C ABI.

EXACT math mode must reproduce the oracle's PORTABLE-mode tallies and final
RNG states bit-for-bit (integer tallies, identical IEEE operations).  FAST
math mode (special-function units) is checked statistically against EXACT
mode with the gate of tests/_stats.py: per bin within 3 sigma of the Monte
Carlo error (the count of |z| > 3 and the chi-square of z consistent with
chance) and the total within 0.5 % relative.  The comparison of FAST mode
with the reference's own kernel at the benchmark sizes is in
test_reference_parity.py.
"""
import os

import numpy as np
import pytest

import _stats
import fiber_sweep
import probe_sweep
import scenarios

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
K = 8388607.0


def gpu_run(mc, nphotons, streams, torch):
    trace, fluence, dets = mc.run(nphotons, maxthreads=streams or None)
    accu = mc._dev['accu'].cpu().numpy().view(np.uint64).copy()
    return accu, mc.rng_states(), mc.run_report


@pytest.mark.parametrize('name', sorted(scenarios.SCENARIOS))
@pytest.mark.parametrize('scheduling', ['static', 'dynamic'])
def test_exact_mode_bit_identical_to_oracle(cuda, lib, oracle, name, scheduling):
    s = scenarios.SCENARIOS[name]
    n, t = s['nphotons'], s['streams']
    mc = scenarios.build_mc(name, scheduling=scheduling)
    ref = oracle.run(mc, n, t, oracle.PORTABLE)
    accu, rng_x, report = gpu_run(mc, n, t, cuda)
    got = oracle.tallies(mc, accu)
    assert set(got) == set(k for k in ref if k in got)
    for k in got:
        assert np.array_equal(got[k], ref[k]), (k, int(got[k].sum()), int(ref[k].sum()))
    assert report['steps'] == ref['steps']
    assert report['packets_done'] == n
    if scheduling == 'static':
        assert np.array_equal(rng_x, ref['rng_x'])
        assert report['threads'] == min(t, n)


def test_dynamic_runs_continue_with_new_packets(cuda, lib, oracle):
    """A second dynamic run simulates packets n..2n-1 (fresh streams)."""
    mc = scenarios.build_mc('c1_line_hg_radial', scheduling='dynamic')
    n = 3000
    a1, _, _ = gpu_run(mc, n, 0, cuda)
    a2, _, _ = gpu_run(mc, n, 0, cuda)
    assert not np.array_equal(a1, a2)
    ref = scenarios.build_mc('c1_line_hg_radial', scheduling='dynamic')
    ref._packets_total = n
    r2 = oracle.run(ref, n, 0, oracle.PORTABLE)
    assert np.array_equal(a2[:r2['accu'].size], r2['accu'])


@pytest.mark.parametrize('name', ['c1_line_hg_radial', 'c3_vox_cylinder'])
def test_dynamic_tallies_independent_of_packets_per_item(cuda, lib, oracle, name):
    """Dynamic scheduling: packet p runs on the stream of (seed, p) whatever
    warp takes it, so the queue granularity cannot change the tallies."""
    s = scenarios.SCENARIOS[name]
    ref = None
    for ppi in (0, 1, 7, 128):
        mc = scenarios.build_mc(name, scheduling='dynamic')
        mc.packets_per_item = ppi
        accu, _, report = gpu_run(mc, s['nphotons'], None, cuda)
        assert report['packets_done'] == s['nphotons']
        if ref is None:
            ref = accu
        assert np.array_equal(accu, ref), ppi


def test_exact_mode_many_streams_bit_identical(cuda, lib, oracle):
    """Full-occupancy launch (many blocks) on the three-layer skin stack."""
    mc = scenarios.build_mc('c2_gk_fluence')
    n, t = 20000, 4096
    ref = oracle.run(mc, n, t, oracle.PORTABLE, nthreads=8)
    accu, rng_x, _ = gpu_run(mc, n, t, cuda)
    assert np.array_equal(accu[:ref['accu'].size], ref['accu'])
    assert np.array_equal(rng_x, ref['rng_x'])


def test_runs_continue_streams(cuda, lib, oracle):
    """Two runs on the same simulator continue the RNG streams (the seed
    state stays on the device), like the reference's persistent
    rng_seeds_x buffer; the oracle chained on the returned states agrees."""
    mc = scenarios.build_mc('semiinf_hg')
    n, t = 600, 16
    a1, x1, _ = gpu_run(mc, n, t, cuda)
    a2, x2, _ = gpu_run(mc, n, t, cuda)
    seeds = mc.host_seeds(t)
    r1 = oracle.run(mc, n, t, oracle.PORTABLE, seeds=seeds)
    r2 = oracle.run(mc, n, t, oracle.PORTABLE, seeds=(r1['rng_x'], seeds[1]))
    assert np.array_equal(a1[:r1['accu'].size], r1['accu'])
    assert np.array_equal(a2[:r2['accu'].size], r2['accu'])


def test_fast_mode_deterministic(cuda, lib):
    a = scenarios.build_mc('c3_vox_cylinder', fast=True)
    b = scenarios.build_mc('c3_vox_cylinder', fast=True)
    ra, _, _ = gpu_run(a, 20000, 2048, cuda)
    rb, _, _ = gpu_run(b, 20000, 2048, cuda)
    assert np.array_equal(ra, rb)


def _batched(mc, nphotons, streams, batches):
    """Per-batch normalized tallies (batches continue the RNG streams)."""
    rows = []
    for _ in range(batches):
        _, _, dets = mc.run(nphotons, maxthreads=streams)
        rows.append(np.asarray(dets.top.raw, dtype=np.float64) / nphotons)
    return np.array(rows)


@pytest.mark.parametrize('name', ['c1_line_hg_radial', 'gk_alpha_1p2_rejection', 'c3_vox_cylinder'])
def test_fast_mode_statistically_equal_to_exact(cuda, lib, name):
    fast = scenarios.build_mc(name, fast=True)
    exact = scenarios.build_mc(name)
    exact._rnginit = 424242
    a = _batched(fast, 200000, 65536, 16)
    b = _batched(exact, 200000, 65536, 16)
    ok, rep = _stats.gate(a, b)
    assert ok, rep
    ta, tb = a.sum(1).mean(), b.sum(1).mean()
    assert abs(ta - tb) / tb < 5e-3


@pytest.mark.parametrize('fast', [False, True])
def test_cuda_mcml_golden_profile(cuda, lib, fast):
    """The reference's validation test SingleLayerLineSourceRadialProfile
    (xopto/mcml/test/validate.py:219-345): radial reflectance against the
    CUDA-MCML profile, pass if |mean relative error| < 0.5 %."""
    from pyxopto_gb300.mcml import mc
    g = np.load(os.path.join(GOLD, 'cuda_mcml_radial.npz'))
    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=float(g['d'][i]), n=float(g['n'][i]), mua=float(g['mua'][i]),
                         mus=float(g['mus'][i]), pf=mc.mcpf.Hg(float(g['g'][i]))) for i in range(3)])
    start, stop, nb = g['axis']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(
        mc.mcdetector.RadialAxis(float(start), float(stop), int(nb)), cosmin=float(g['cosmin'][0])))
    opts = [mc.mcoptions.McUseNativeMath(True)] if fast else []
    sim = mc.Mc(layers, mc.mcsource.Line(), det, options=opts, rnginit=5)
    sim.rmax = float(g['rmax'][0])
    _, _, res = sim.run(10_000_000)
    rel = (res.top.reflectance - g['reflectance']) / g['reflectance'] * 100.0
    assert abs(np.mean(rel)) < 0.5, np.mean(rel)


def test_rng_dump_matches_oracle(cuda, lib, oracle):
    from pyxopto_gb300.mcml import mc
    sim = scenarios.build_mc('c1_line_hg_radial')
    out = sim.rng_test(5000, 18446741578333584324, 4294966893)
    assert np.array_equal(out, oracle.rng_dump(18446741578333584324, 4294966893, 5000))


@pytest.mark.parametrize('scheduling', ['static', 'dynamic'])
def test_trace_bit_identical_to_oracle(cuda, lib, oracle, scheduling):
    from pyxopto_gb300.mcml import mc
    spec = dict(scenarios.SCENARIOS['c1_line_hg_radial'])
    sim = scenarios.build_mc(spec, scheduling=scheduling)
    sim._trace = mc.mctrace.Trace(maxlen=64, options=mc.mctrace.Trace.TRACE_ALL)
    n, t = 300, 32
    ref = oracle.run(sim, n, t, oracle.PORTABLE)
    tr, _, _ = sim.run(n, maxthreads=t)
    off, cnt = sim._flt.find(sim._trace)
    ioff, icnt = sim._int.find(sim._trace)
    assert np.array_equal(tr.n, ref['int'][ioff:ioff + icnt])
    got = np.ascontiguousarray(tr.data).view(np.float32).reshape(-1)
    assert np.array_equal(got, ref['float'][off:off + cnt])
    assert tr.n.min() >= 1


@pytest.mark.parametrize('double', [False, True])
def test_cuda_mcml_fiber_sweep(cuda, lib, double):
    """The reference's validation tests SingleLayerUniformFiberRadial and
    DoubleLayerUniformFiberRadial (xopto/mcml/test/validate.py:348-511,
    692-866): fibre reflectance of a 20 x 20 (mua, mus') sweep at 5
    source-detector separations against CUDA-MCML, pass if |mean relative
    error| < 0.5 % (1e6 packets per point here, 1e7 in the reference)."""
    data = fiber_sweep.load(double)
    sim = fiber_sweep.build(data, fast=True)
    refl, _ = fiber_sweep.run(sim, data, 1_000_000)
    err = fiber_sweep.relative_error(data, refl)
    assert abs(err.mean()) < 0.5, err.mean()
    assert np.median(np.abs(err)) < 3.0, np.median(np.abs(err))


@pytest.mark.parametrize('key', probe_sweep.KEYS)
def test_linear_probe_sweep(cuda, lib, key):
    """The reference's linear fibre-probe validation tests
    (xopto/mcml/test/validate.py:1227-1758) on every fifth sweep point with
    1e7 packets per point, as the reference runs them: the fibre source in
    fibre 0 of a LinearArray probe face, the reflectance of fibres 1.. of a
    LinearArray detector.  The reference passes at |mean relative error| <
    0.5 % over its full sweep; on the subset the noise of the mean is about
    0.3 %, so the bound here is 1 %.  The ratio of the summed reflectances
    of each fibre must agree within 3 %: both sides are Monte Carlo
    estimates, and on the 80-point Gegenbauer subset the farthest fibre's
    sum carries about 1 % noise."""
    data = probe_sweep.load(key)
    sim = probe_sweep.build(data, fast=True)
    refl, ref, _ = probe_sweep.run(sim, data, 10_000_000, stride=5)
    err = probe_sweep.relative_error(refl, ref)
    assert abs(err.mean()) < 1.0, err.mean()
    ratio = refl.sum(axis=0) / ref.sum(axis=0)
    assert np.all(np.abs(ratio - 1.0) < 0.03), ratio


SV_SCENARIOS = sorted(n for n, s in scenarios.SCENARIOS.items() if s.get('sampling_volume'))


def _sv_expected(oracle, sim, sv, tr):
    cfg = sv.pack(sim)
    cfg.max_events, cfg.num_packets = tr.maxlen, len(tr)
    accu, total, status = oracle.sampling_volume(cfg, tr.n, np.ascontiguousarray(tr.data).view(np.float32))
    assert status == 0
    data = np.reshape(accu.astype(np.float64), sv.shape) * (1.0 / (sv.k * sv._multiplier()))
    return data, float(total[0]) / sv.k


@pytest.mark.parametrize('name', SV_SCENARIOS)
@pytest.mark.parametrize('scheduling', ['static', 'dynamic'])
def test_sampling_volume_bit_identical_to_oracle(cuda, lib, oracle, name, scheduling):
    """Mc.sampling_volume on the GPU equals the oracle's walk (pinned to the
    reference's SamplingVolume kernel) on the same trace, tally for tally;
    under static scheduling the trace itself is the oracle's."""
    s = scenarios.SCENARIOS[name]
    sim = scenarios.build_mc(name, scheduling=scheduling)
    tr, _, _ = sim.run(s['nphotons'], maxthreads=s['streams'])
    if scheduling == 'static':
        ref = oracle.run(sim, s['nphotons'], s['streams'], oracle.PORTABLE)
        ioff, icnt = sim._int.find(sim.trace)
        assert np.array_equal(tr.n, ref['int'][ioff:ioff + icnt])
    sv = scenarios._sampling_volume(sim, s['sampling_volume'])
    out = sim.sampling_volume(tr, sv)
    assert out is sv
    data, weight = _sv_expected(oracle, sim, sv, tr)
    assert np.array_equal(out.data, data)
    assert out.weight == weight
    assert np.count_nonzero(out.data) > 100


def test_sampling_volume_large_trace(cuda, lib, oracle):
    """A 20,000-packet, 500-event trace of the FAST dynamic kernel, filtered
    to the packets that leave through the top within 0.5 mm of the source
    (the reference's sampling-volume example), then a 100^3 sampling volume:
    bit-identical to the oracle, and a second call accumulates."""
    from pyxopto_gb300.mcml import mc
    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=0.0, n=1.45, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0)),
        mc.mclayer.Layer(d=1e-2, n=1.33, mua=2e2, mus=250e2, pf=mc.mcpf.Hg(0.9)),
        mc.mclayer.Layer(d=0.0, n=1.45, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0))])
    trace = mc.mctrace.Trace(maxlen=500, filter=mc.mctrace.Filter(
        z=(-1e-9, 1e-9), pz=(-1.0, -0.2), r=(0.0, 5e-4, (0.0, 0.0))))
    sim = mc.Mc(layers, mc.mcsource.Line(), trace=trace,
                options=[mc.mcoptions.McUseNativeMath(True), mc.mcoptions.McScheduling('dynamic')],
                rnginit=3)
    sim.rmax = 1e-2
    tr, _, _ = sim.run(20000)
    assert len(tr) > 500
    A = mc.mcsv.Axis
    sv = mc.mcsv.SamplingVolume(A(-1e-3, 1e-3, 100), A(-1e-3, 1e-3, 100), A(0.0, 2e-3, 100))
    sim.sampling_volume(tr, sv)
    data, weight = _sv_expected(oracle, sim, sv, tr)
    assert np.array_equal(sv.data, data) and sv.weight == weight
    sim.sampling_volume(tr, sv)
    assert np.array_equal(sv.data, 2.0 * data)


def test_sfdi_30deg_variable_na(cuda, lib):
    """The reference's SFDI validation test (xopto/mcml/test/validate.py:
    867-1050) on every fourth detector NA from index 4, 1e7 packets per NA
    as the reference runs it: the per-NA mean |relative amplitude error| and
    mean |phase error| must stay below its bounds of 2.5 % and 0.025 rad."""
    import sfdi_sweep
    data = sfdi_sweep.load()
    idx = list(range(4, data['na'].size, 4))
    amp, ph, _ = sfdi_sweep.run(data, 10_000_000, idx)
    ea, ep = sfdi_sweep.errors(data, idx, amp, ph)
    assert ea.max() < 0.025, ea
    assert ep.max() < 0.025, ep


@pytest.mark.parametrize('fast', [False, True])
def test_cuda_mcml_golden_profile_voxelized(cuda, lib, fast):
    """The voxelized simulator's version of SingleLayerLineSourceRadialProfile
    (xopto/mcvox/test/validate.py:213-356): the layer as one voxel spanning
    +-2 rmax, radial reflectance against the CUDA-MCML profile, pass if
    |mean relative error| < 0.5 %."""
    from pyxopto_gb300.mcvox import mc
    g = np.load(os.path.join(GOLD, 'cuda_mcml_radial.npz'))
    rmax = float(g['rmax'][0])
    A = mc.mcgeometry.Axis
    vox = mc.mcgeometry.Voxels(A(-2.0 * rmax, 2.0 * rmax, 1), A(-2.0 * rmax, 2.0 * rmax, 1),
                               A(0.0, float(g['d'][1]), 1))
    mats = [mc.mcmaterial.Material(n=float(g['n'][i]), mua=float(g['mua'][i]), mus=float(g['mus'][i]),
                                   pf=mc.mcpf.Hg(float(g['g'][i]))) for i in range(2)]
    start, stop, nb = g['axis']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(
        mc.mcdetector.RadialAxis(float(start), float(stop), int(nb)), cosmin=float(g['cosmin'][0])))
    opts = [mc.mcoptions.McUseNativeMath(True)] if fast else []
    sim = mc.Mc(vox, mats, mc.mcsource.Line(), det, options=opts, rnginit=7)
    sim.rmax = rmax
    sim.voxels.material[...] = 1
    _, _, res = sim.run(10_000_000)
    rel = (res.top.reflectance - g['reflectance']) / g['reflectance'] * 100.0
    assert abs(np.mean(rel)) < 0.5, np.mean(rel)


@pytest.mark.parametrize('double', [False, True])
def test_cuda_mcml_fiber_sweep_voxelized(cuda, lib, double):
    """The voxelized simulator's SingleLayerUniformFiberRadial and
    DoubleLayerUniformFiberRadial (xopto/mcvox/test/validate.py:357-536,
    730-925; the two-layer sample as 85 voxels of 0.1 mm in depth) against
    the CUDA-MCML fibre reflectances, pass if |mean relative error| < 0.5 %
    (1e6 packets per point here, 1e7 in the reference)."""
    data = fiber_sweep.load(double)
    sim = fiber_sweep.build_vox(data, fast=True)
    refl, _ = fiber_sweep.run(sim, data, 1_000_000)
    err = fiber_sweep.relative_error(data, refl)
    assert abs(err.mean()) < 0.5, err.mean()
    assert np.median(np.abs(err)) < 3.0, np.median(np.abs(err))


def test_uniformfiber_trace_matches_radial_detector(cuda, lib):
    """The reference's SingleLayerUniformFiberTrace test
    (xopto/mcml/test/validate.py:1059-1226): 1e6 packets of a UniformFiber
    source with a 100-event trace; the reflectance rebuilt from the terminal
    trace events (z <= 0, |pz| >= cosmin) equals the Radial detector's in
    every ring within 0.1 %, for five (mua, mus') points."""
    from pyxopto_gb300.mcml import mc
    from pyxopto_gb300.mcml.mcutil import fiber
    d = np.load(os.path.join(GOLD, 'uniformfiber_trace.npz'))
    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=float(d['d'][i]), n=float(d['n'][i]), mua=0.0, mus=0.0,
                         pf=mc.mcpf.Hg(float(d['g'][i]))) for i in range(3)])
    dcore, dclad, ncore, na = (float(v) for v in d['fiber'])
    source = mc.mcsource.UniformFiber(fiber.MultimodeFiber(dcore, dclad, ncore, na))
    start, stop, nb = d['axis']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(
        mc.mcdetector.RadialAxis(float(start), float(stop), int(nb)), cosmin=float(d['cosmin'][0])))
    sim = mc.Mc(layers, source, det, mc.mctrace.Trace(maxlen=int(d['maxlen'][0])),
                options=[mc.mcoptions.McUseNativeMath(True)], rnginit=11)
    sim.rmax = float(d['rmax'][0])
    top = sim.detectors.top
    edges, nr, cosmin = top.edges, top.n, top.cosmin
    dr = edges[1] - edges[0]
    rings = np.pi * (edges[1:] ** 2 - edges[:-1] ** 2)
    nphotons = 1_000_000
    g1 = float(d['g'][1])
    for mua, musr in zip(d['mua'], d['musr']):
        sim.layers[1].mua = float(mua)
        sim.layers[1].mus = float(musr) / (1.0 - g1)
        tr, _, res = sim.run(nphotons)
        term = np.minimum(tr.n - 1, tr.maxlen - 1)
        last = tr.data[np.arange(nphotons), term]
        rind = np.minimum(np.floor(np.sqrt(last['x'] ** 2 + last['y'] ** 2) / dr), nr - 1).astype(int)
        ok = (last['z'] <= 0.0) & (np.abs(last['pz']) >= cosmin)
        refl_trace = np.bincount(rind[ok], weights=last['w'][ok].astype(np.float64), minlength=nr)
        refl_trace = refl_trace / (nphotons * rings)
        refl = res.top.reflectance
        mask = refl != 0
        assert not np.any((refl == 0) & (refl_trace != 0))
        if mask.any():      # no reflectance at all for the purely absorbing point
            err = np.abs(refl_trace[mask] - refl[mask]) / refl[mask]
            assert err.max() < 1e-3, (mua, musr, err.max())


def test_cuda_mcml_fiber_sweep_cartesian(cuda, lib):
    """The reference's SingleLayerUniformFiberCartesian test
    (xopto/mcml/test/validate.py:514-690): the fibre sweep with a Cartesian
    detector resampled by Cartesian.radial, against the CUDA-MCML fibre
    reflectances; pass if |mean relative error| < 0.5 % (1e6 packets per
    point here, 1e7 in the reference)."""
    data = fiber_sweep.load()
    sim, raxis = fiber_sweep.build_cartesian(data, fast=True)
    refl, _ = fiber_sweep.run(sim, data, 1_000_000, raxis=raxis)
    err = fiber_sweep.relative_error(data, refl)
    assert abs(err.mean()) < 0.5, err.mean()


def test_run_helpers(cuda, lib):
    """RunMinWeightTop and McRunHelper (xopto/mcml/mcrun) drive Mc.run:
    batches accumulate until the top detector holds the asked weight, and a
    helper subclass updates the layers before each of its runs."""
    from pyxopto_gb300.mcml import mc, mcrun
    sim = scenarios.build_mc('c1_line_hg_radial', scheduling='dynamic')
    runner = mcrun.RunMinWeightTop(min_weight=500.0, batch_size=20_000)
    trace, fluence, det = runner.run(sim)
    assert runner.weight >= 500.0 and runner.n % 20_000 == 0
    assert det.top.nphotons == runner.n

    class Helper(mcrun.McRunHelper):
        def create_layers(self):
            return mc.mclayer.Layers([
                mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.8)),
                mc.mclayer.Layer(d=float('inf'), n=1.4, mua=100.0, mus=1e4, pf=mc.mcpf.Hg(0.8)),
                mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.8))])

        def create_detectors(self):
            return mc.mcdetector.Detectors(top=mc.mcdetector.Total())

        def update_layers(self):
            self.mc_obj.layers[1].mua *= 2.0

    h = Helper(options=[mc.mcoptions.McUseNativeMath(True)])
    res = h.run_batch(3, 100_000)
    totals = [float(np.sum(r['detectors']['reflectance'])) for r in res]
    assert [r['index'] for r in res] == [0, 1, 2]
    assert totals[0] > totals[1] > totals[2] > 0.0     # more absorption, less reflectance


def test_fast_voxel_fluence_statistically_equal_to_exact(cuda, lib):
    """The fluence FAST mode deposits in a voxelized medium agrees with EXACT
    mode (bit-identical to the reference kernel): per depth slice within the
    3-sigma gate over 20 batches of 4e5 packets (the slices share packets;
    the gate takes their covariance from the batches), and the total within
    0.5 %."""
    spec = dict(scenarios.SCENARIOS['c3_vox_cylinder'])
    fast = scenarios.build_mc(spec, fast=True, scheduling='dynamic')
    exact = scenarios.build_mc(spec, scheduling='dynamic')
    fast._rnginit, exact._rnginit = 1234, 2011

    def batches(mc):
        rows = []
        for _ in range(20):
            _, flu, _ = mc.run(400_000)
            raw = np.asarray(flu.raw, dtype=np.float64)
            rows.append(raw.reshape(raw.shape[0], -1).sum(1) / 4e5)
        return np.array(rows)
    fa, ea = batches(fast), batches(exact)
    ok, rep = _stats.gate(fa, ea)
    assert ok, rep
    assert abs(fa.sum(1).mean() / ea.sum(1).mean() - 1.0) < 5e-3


@pytest.mark.parametrize('name', ['c3_vox_skin_vessel', 'vox_sphere_mismatch'])
def test_phased_voxel_loop_keeps_every_packet_unchanged(cuda, lib, name):
    """The plain FAST voxel kernel defers a lane's wall steps until half of
    the warp's lanes wait for one (phased loop); each packet still runs the
    same operations in the same order as in the unphased loop, which the
    feature kernel keeps (chosen here by a step limit that is never reached):
    fluence and detector tallies and the step count are the same integers."""
    n = 2_000_000 if name == 'c3_vox_skin_vessel' else 500_000
    out = []
    for limit in (0, 1 << 40):
        mc = scenarios.build_mc(name, fast=True, scheduling='dynamic')
        mc._rnginit = 31
        mc.max_steps_per_packet = limit
        _, flu, det = mc.run(n)
        out.append((np.asarray(flu.raw).copy(), np.asarray(det.top.raw).copy(),
                    np.asarray(det.bottom.raw).copy(), mc.run_report['steps']))
    (fa, ta, ba, sa), (fb, tb, bb, sb) = out
    assert sa == sb
    assert np.array_equal(ta, tb) and np.array_equal(ba, bb)
    assert np.array_equal(fa, fb)


def test_box_stepping_reflects_and_refracts_like_the_wall_walk(cuda, lib):
    """Free flight and box stepping where the faces of large homogeneous
    cubes meet a refractive-index step (a sphere of n 1.6 in a cube of
    n 1.33 under air), against the wall-by-wall walk in the same FAST
    kernels: depth profile, 0.4 mm voxels, the deposits inside and outside
    the sphere and the detector totals within the 3-sigma gate."""
    from pyxopto_gb300.mcvox import mcoptions
    name, nb, n = 'vox_sphere_mismatch', 16, 400_000
    spec = scenarios.ALL[name]
    inside = scenarios.voxel_layout(spec['grid'], spec['layout']).reshape(-1) == 2
    fly = scenarios.build_mc(name, fast=True, scheduling='dynamic')
    walk = scenarios.build_mc(name, fast=True, scheduling='dynamic')
    walk._mc_options.append(mcoptions.McVoxelFreeFlight(False))
    walk._rnginit = 977

    def batches(mc):
        rows, tots, steps = [], [], 0
        for _ in range(nb):
            _, flu, det = mc.run(n)
            raw = np.asarray(flu.raw, dtype=np.float64).reshape(-1)
            rows.append(raw)
            tots.append([float(det.top.raw.sum()), float(det.bottom.raw.sum()),
                         raw[inside].sum(), raw[~inside].sum()])
            steps += mc.run_report['steps']
        return np.array(rows) / n, np.array(tots) / n, steps
    fa, ta, sa = batches(fly)
    wa, tw, sw = batches(walk)
    depth = lambda f: f.reshape(nb, 64, -1).sum(2)
    coarse = lambda f: f.reshape(nb, 8, 8, 8, 8, 8, 8).sum(axis=(2, 4, 6)).reshape(nb, -1)
    for what, a, b in (('depth', depth(fa), depth(wa)), ('coarse', coarse(fa), coarse(wa)),
                       ('totals', ta, tw)):
        keep = (b.mean(0) > 0) & (b.std(0, ddof=1) / np.sqrt(nb) < 0.2 * b.mean(0))
        ok, rep = _stats.gate(a[:, keep], b[:, keep])
        assert ok, (what, rep)
    assert sa < 0.8 * sw, (sa, sw)


def _radius_reference(mat, cap):
    """Largest k <= cap whose cube of voxels within Chebyshev distance k lies
    inside the grid and holds one material (brute force over k)."""
    from scipy import ndimage
    nz, ny, nx = mat.shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing='ij')
    edge = np.minimum.reduce([x, y, z, nx - 1 - x, ny - 1 - y, nz - 1 - z])
    out = np.zeros(mat.shape, np.int64)
    m = mat.astype(np.int64)
    for k in range(1, cap + 1):
        hi = ndimage.maximum_filter(m, size=2 * k + 1, mode='nearest')
        lo = ndimage.minimum_filter(m, size=2 * k + 1, mode='nearest')
        ok = (hi == m) & (lo == m) & (edge >= k)
        out[ok] = k
    return out


def test_voxel_radius_table_matches_brute_force(cuda, lib):
    """mcgb_voxel_radius (the free-flight table) against a brute-force
    search on a grid with layers, a sphere and a thin plate."""
    import ctypes as C
    from pyxopto_gb300 import _lib
    torch = cuda
    nz, ny, nx = 24, 30, 40
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing='ij')
    mat = np.ones((nz, ny, nx), np.uint8)
    mat[z < 3] = 2
    mat[(x - 20) ** 2 + (y - 14) ** 2 + (z - 12) ** 2 <= 36] = 3
    mat[(x == 33) & (z > 5)] = 4
    for cap in (3, 31):
        dev = torch.from_numpy(mat.reshape(-1).copy()).cuda()
        rad = torch.full_like(dev, 77)
        shape = (C.c_int32 * 3)(nx, ny, nz)
        _lib.check(lib.mcgb_voxel_radius(C.c_void_p(dev.data_ptr()), shape, C.c_void_p(rad.data_ptr()),
                                         cap, None))
        got = rad.cpu().numpy().reshape(mat.shape).astype(np.int64)
        assert np.array_equal(got, _radius_reference(mat, cap)), cap


@pytest.mark.parametrize('rmax', [None, 1.5e-3])
def test_voxel_free_flight_statistically_equal_to_wall_walk(cuda, lib, rmax):
    """Free flight (the FAST-math default in voxelized media) against the
    reference's wall-by-wall walk in the same FAST kernels, on the 200^3
    skin and vessel grid: depth profile, 1 mm^3 voxels and the detector
    totals within the 3-sigma gate; free flight takes far fewer steps.  With
    a finite rmax the packets must end where the walk ends them (no fluence
    beyond the voxel that crosses the rmax sphere)."""
    from pyxopto_gb300.mcvox import mcoptions
    name, nb, n = 'c3_vox_skin_vessel', 16, 1_000_000
    fly = scenarios.build_mc(name, fast=True, scheduling='dynamic')
    walk = scenarios.build_mc(name, fast=True, scheduling='dynamic')
    walk._mc_options.append(mcoptions.McVoxelFreeFlight(False))
    walk._rnginit = 4321
    if rmax is not None:
        fly.rmax = walk.rmax = rmax

    def batches(mc):
        rows, tops, steps = [], [], 0
        for _ in range(nb):
            _, flu, det = mc.run(n)
            raw = np.asarray(flu.raw, dtype=np.float64)
            rows.append(raw)
            tops.append([float(det.top.raw.sum()), float(det.bottom.raw.sum())])
            steps += mc.run_report['steps']
        return np.array(rows) / n, np.array(tops) / n, steps
    fa, ta, sa = batches(fly)
    wa, tw, sw = batches(walk)
    depth = lambda f: f.reshape(nb, 200, -1).sum(2)
    coarse = lambda f: f.reshape(nb, 10, 20, 10, 20, 10, 20).sum(axis=(2, 4, 6)).reshape(nb, -1)
    for what, a, b in (('depth', depth(fa), depth(wa)), ('coarse', coarse(fa), coarse(wa)),
                       ('totals', ta, tw)):
        keep = (b.mean(0) > 0) & (b.std(0, ddof=1) / np.sqrt(nb) < 0.2 * b.mean(0))
        ok, rep = _stats.gate(a[:, keep], b[:, keep])
        assert ok, (what, rep)
    if rmax is not None:
        # no deposit beyond the voxel that crosses the rmax sphere (centred
        # on the beam's origin): beyond rmax + 1.5 voxel diagonals all is 0
        c = (np.arange(200) + 0.5) * 5e-5
        zc, yc, xc = np.meshgrid(c, c - 5e-3, c - 5e-3, indexing='ij')
        far = np.sqrt(xc ** 2 + yc ** 2 + zc ** 2).reshape(-1) > rmax + 1.5 * np.sqrt(3) * 5e-5
        assert not fa.reshape(nb, -1)[:, far].any() and not wa.reshape(nb, -1)[:, far].any()
    assert sa < (0.8 if rmax is None else 0.95) * sw, (sa, sw)
