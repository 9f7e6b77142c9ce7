"""Batched engine: CPU restatement sanity, and on the GPU bit-identity with
the oracle, independence of the tallies from the launch shape, CUDA-graph
replay and statistical agreement with plain layered-medium runs."""
import numpy as np
import pytest

import scenarios


def small_batch(num=24, seed=3, packets=(200, 600)):
    from pyxopto_gb300.batched import BatchedMc
    sims = BatchedMc.sample_sims(num, seed=seed, packets=packets)
    sims['thickness'][::3] = 2e-3                    # a few finite slabs
    sims['n_below'][::3] = 1.33
    return sims


def test_batched_oracle_matches_layered_oracle_statistically(oracle, lib):
    """A batch simulation and a layered run of the same layer agree within
    the Monte Carlo error of the total reflectance."""
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.mcml import mc
    sims = {'mua': [50.0], 'mus': [6000.0], 'g': [0.8], 'n': [1.4], 'thickness': [np.inf],
            'num_packets': [4000]}
    b = BatchedMc(sims, raxis=mc.mcdetector.Axis(0.0, 3e-3, 30), fast=False)
    tb, _ = oracle.batched_run(b, nthreads=4)
    spec = dict(medium='mcml', layers=[dict(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=['Hg', 0.0]),
                                       dict(d=np.inf, n=1.4, mua=50.0, mus=6000.0, pf=['Hg', 0.8]),
                                       dict(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=['Hg', 0.0])],
                source=dict(type='Line'), detectors=dict(top=dict(type='Radial', axis=[0.0, 3e-3, 30])),
                rnginit=5)
    m = scenarios.build_mc(spec)
    r = oracle.run(m, 4000, 64, oracle.PORTABLE, nthreads=4)
    ra, rb = tb.sum() / 8388607.0 / 4000, r['top'].sum() / 8388607.0 / 4000
    sigma = np.sqrt(2 * ra * (1 - ra) / 4000)
    assert abs(ra - rb) < 4 * sigma


@pytest.mark.gpu
def test_batched_exact_bit_identical_to_oracle(cuda, lib, oracle):
    from pyxopto_gb300.batched import BatchedMc
    b = BatchedMc(small_batch(), fast=False)
    ref, steps = oracle.batched_run(b, nthreads=8)
    got = b.run_raw()
    assert np.array_equal(got, ref)
    assert b.last_report['steps'] == steps
    assert b.last_report['packets'] == int(b.packets.sum())


@pytest.mark.gpu
def test_batched_tallies_independent_of_launch_shape(cuda, lib):
    from pyxopto_gb300.batched import BatchedMc
    b = BatchedMc(small_batch(64, packets=(500, 5000)), fast=True)
    a = b.run_raw(block_size=128, packets_per_item=256)
    for bs, it, bps in [(64, 32, 0), (256, 1024, 0), (128, 64, 1)]:
        assert np.array_equal(b.run_raw(block_size=bs, packets_per_item=it, blocks_per_sm=bps), a)


@pytest.mark.gpu
def test_batched_graph_replay(cuda, lib):
    from pyxopto_gb300.batched import BatchedMc
    b = BatchedMc(small_batch(48), fast=True)
    plain = b.run_raw()
    g1 = b.run_raw(graph=True)
    g2 = b.run_raw(graph=True)
    assert np.array_equal(plain, g1) and np.array_equal(g1, g2)
    # new parameters flow into the captured graph
    sims = small_batch(48, seed=9)
    b.set_sims(sims)
    g3 = b.run_raw(graph=True)
    assert np.array_equal(g3, b.run_raw())
    assert not np.array_equal(g3, g1)


@pytest.mark.gpu
def test_batched_matches_plain_runs(cuda, lib):
    """Each batched simulation is statistically the layered simulator's run
    of the same layer (fast math both)."""
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.mcml import mc
    sims = BatchedMc.sample_sims(6, seed=11, packets=(400000, 400001))
    b = BatchedMc(sims, raxis=mc.mcdetector.Axis(0.0, 3e-3, 30), fast=True)
    raw = b.run_raw().astype(np.float64) / 8388607.0
    for i in range(6):
        layers = mc.mclayer.Layers([
            mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0)),
            mc.mclayer.Layer(d=np.inf, n=float(np.float32(sims['n'][i])),
                             mua=float(np.float32(sims['mua'][i])),
                             mus=float(np.float32(sims['mus'][i])),
                             pf=mc.mcpf.Hg(float(np.float32(sims['g'][i])))),
            mc.mclayer.Layer(d=0.0, n=1.0, mua=0.0, mus=0.0, pf=mc.mcpf.Hg(0.0))])
        det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(mc.mcdetector.Axis(0.0, 3e-3, 30)))
        m = mc.Mc(layers, mc.mcsource.Line(), det, options=[mc.mcoptions.McUseNativeMath(True)],
                  rnginit=100 + i)
        _, _, d = m.run(400000)
        # total diffuse reflectance per packet: relative MC error ~0.2 % here
        ra = raw[i].sum() / 400000
        rb = d.top.raw.sum() / 400000
        assert abs(ra - rb) / rb < 0.01, (i, ra, rb)


@pytest.mark.gpu
def test_autotune_picks_a_candidate(cuda, lib, tmp_path):
    from pyxopto_gb300.batched import BatchedMc
    b = BatchedMc(small_batch(128, packets=(2000, 20000)), fast=True)
    best = b.autotune(block_sizes=(64, 128), items=(64, 256), cache=str(tmp_path / 'a.json'))
    assert best['block_size'] in (64, 128) and best['packets_per_item'] in (64, 256)
    again = b.autotune(block_sizes=(64, 128), items=(64, 256), cache=str(tmp_path / 'a.json'))
    assert again['block_size'] == best['block_size']
