"""The shipped path against the reference's own kernel at the benchmark
configurations.

The path every user and the benchmark take (Mc.run with FAST math and
dynamic scheduling) is compared with the reference's McKernel
(xopto/mcml/kernel/mcml.template.c:346-824, xopto/mcvox/kernel/
mcvox.template.c:548-1048), rendered by the reference's own plugins and
compiled for the CPU (oracle/_ref/, built by __graft_entry__.build()), run
on the reference's seeds (clrng.Random().seeds(4096, 1), stored in
tests/golden/ref_seeds.npz) on every host core.

Both sides run as independent batches: the reference's 4096 streams are
split into 16 groups of 256, and the GPU runs 16 consecutive Mc.run calls
(each continues with new packets).  Every tally is then held to the
spec bar through tests/_stats.gate: per bin within 3 sigma of the
Monte Carlo error (the count of |z| > 3 and the chi-square of z consistent
with chance, p > 1e-3), and total reflectance within 0.5 % relative at 1e8
packets.
"""
import os

import numpy as np
import pytest

import _stats
import mcoracle
import render_ref
import scenarios

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
BATCHES = 16


def _seeds():
    d = np.load(os.path.join(GOLD, 'ref_seeds.npz'))
    return d['x'], d['a']


def _need_reference_build(name):
    so = os.path.join(render_ref.REF_DIR, name + '.so')
    assert os.path.exists(so), ('reference CPU build {} is missing: run '
                                '__graft_entry__.build() first'.format(so))


def reference_batches(name, nphotons, keys):
    """Per-batch tallies of the reference build: dict key -> (16, bins)."""
    _need_reference_build(name)
    x, a = _seeds()
    per = len(x) // BATCHES
    rows = {k: [] for k in keys}
    threads = os.cpu_count() or 1
    for k in range(BATCHES):
        sl = slice(k * per, (k + 1) * per)
        out = render_ref.run_ref(name, nphotons // BATCHES, per, (x[sl], a[sl]), nthreads=threads)
        for key in keys:
            rows[key].append(out[key].astype(np.float64))
    return {k: _stats.per_packet(v, nphotons // BATCHES) for k, v in rows.items()}


def gpu_batches(name, nphotons, keys):
    """Per-batch tallies of Mc.run (FAST math, dynamic scheduling)."""
    mc = scenarios.build_mc(name, fast=True, scheduling='dynamic')
    rows = {k: [] for k in keys}
    for _ in range(BATCHES):
        mc.run(nphotons // BATCHES)
        accu = mc._dev['accu'].cpu().numpy().view(np.uint64)
        t = mcoracle.tallies(mc, accu)
        assert mc.run_report['packets_done'] == nphotons // BATCHES
        for key in keys:
            rows[key].append(t[key].astype(np.float64))
    return {k: _stats.per_packet(v, nphotons // BATCHES) for k, v in rows.items()}


def _assert_gate(a, b, what):
    ok, rep = _stats.gate(a, b)
    _stats.record(what, rep)
    assert ok, (what, rep)
    return rep


def test_c1_radial_profile_per_bin_3sigma(cuda, lib):
    """The 10 mm slab at its full 1e6 packets: the 50 radial bins, the total
    and the specular reflectance."""
    keys = ['top', 'specular']
    ref = reference_batches('c1_slab_hg_radial', 1_000_000, keys)
    gpu = gpu_batches('c1_slab_hg_radial', 1_000_000, keys)
    _assert_gate(gpu['top'], ref['top'], 'radial bins')
    _assert_gate(gpu['top'].sum(1, keepdims=True), ref['top'].sum(1, keepdims=True), 'total')
    # the specular reflectance of a normal Line source is deterministic
    assert np.allclose(gpu['specular'], ref['specular'], rtol=1e-6, atol=0.0)


def test_c1_total_reflectance_1e8_within_half_percent(cuda, lib):
    """Spec bar: total diffuse reflectance at 1e8 packets within 0.5 %
    relative of the reference build at 1e8 packets, and within 3 sigma."""
    keys = ['top']
    ref = reference_batches('c1_slab_hg_radial', 100_000_000, keys)
    gpu = gpu_batches('c1_slab_hg_radial', 100_000_000, keys)
    rr, rg = ref['top'].sum(1), gpu['top'].sum(1)
    assert abs(rg.mean() / rr.mean() - 1.0) < 5e-3, (rg.mean(), rr.mean())
    _assert_gate(rg[:, None], rr[:, None], 'total diffuse reflectance')


def _rebin(flu, shape, factor):
    """(batches, nz*ny*nx) -> (batches, cells) summed over factor^3 blocks."""
    nz, ny, nx = shape
    f = np.asarray(flu).reshape(len(flu), nz // factor, factor, ny // factor, factor,
                                nx // factor, factor)
    return f.sum(axis=(2, 4, 6)).reshape(len(flu), -1)


def _populated(ref, rel_se=0.2):
    """Cells whose reference mean is resolved to better than rel_se."""
    m = ref.mean(0)
    se = ref.std(0, ddof=1) / np.sqrt(len(ref))
    return (m > 0) & (se < rel_se * m)


def _fluence_checks(name, n_ref, n_gpu, shape, extra=None):
    keys = ['top', 'bottom', 'specular', 'fluence']
    ref = reference_batches(name, n_ref, keys)
    gpu = gpu_batches(name, n_gpu, keys)
    nz, ny, nx = shape
    reports = {}
    fr, fg = ref['fluence'], gpu['fluence']
    # depth profile (sum over x and y)
    dr = fr.reshape(BATCHES, nz, ny * nx).sum(2)
    dg = fg.reshape(BATCHES, nz, ny * nx).sum(2)
    keep = _populated(dr)
    assert keep.sum() > 0.9 * nz
    reports['depth'] = _assert_gate(dg[:, keep], dr[:, keep], 'depth profile')
    # coarse voxels, 10 x 10 x 10 cells over the grid
    f = nx // 10
    cr, cg = _rebin(fr, shape, f), _rebin(fg, shape, f)
    keep = _populated(cr)
    assert keep.sum() > 500
    reports['coarse'] = _assert_gate(cg[:, keep], cr[:, keep], 'coarse voxels')
    if extra:
        reports.update(extra(fr, fg))
    # total deposit and the detector totals
    reports['deposit'] = _assert_gate(fg.sum(1, keepdims=True), fr.sum(1, keepdims=True), 'total deposit')
    for k in ('top', 'bottom'):
        reports[k] = _assert_gate(gpu[k], ref[k], k)
    assert abs(gpu['top'].mean() / ref['top'].mean() - 1.0) < 5e-3
    assert np.allclose(gpu['specular'], ref['specular'], rtol=1e-5, atol=0.0)
    return reports


def test_c2_fluence_grid_against_reference(cuda, lib):
    """The three-layer skin stack on its 100^3 fluence grid: the GPU at 1e8
    packets against the reference build at 1e7, per depth slice, per 1 mm^3
    coarse voxel, and the top, bottom and specular totals."""
    _fluence_checks('c2_skin_gk_fluence', 10_000_000, 100_000_000, (100, 100, 100))


def test_c3_voxel_fluence_against_reference(cuda, lib):
    """The skin and vessel voxels on their 200^3 grid: the GPU at 1e8 packets
    against the reference build at 1e7, per depth slice, per 1 mm^3 coarse
    voxel, on the x-z plane through the vessel (summed over y, 0.25 mm
    cells), and the totals."""
    shape = (200, 200, 200)

    def xz_plane(fr, fg):
        def proj(f):
            p = np.asarray(f).reshape(BATCHES, 200, 200, 200).sum(2)        # (z, x)
            return p.reshape(BATCHES, 40, 5, 40, 5).sum(axis=(2, 4)).reshape(BATCHES, -1)
        pr, pg = proj(fr), proj(fg)
        keep = _populated(pr)
        assert keep.sum() > 800
        return {'xz': _assert_gate(pg[:, keep], pr[:, keep], 'x-z plane')}

    _fluence_checks('c3_vox_skin_vessel', 10_000_000, 100_000_000, shape, extra=xz_plane)


def test_batched_engine_against_reference(cuda, lib):
    """The batched engine (FAST math, one persistent launch) against the
    reference build of the same single-layer simulation: 16 copies of the
    simulation of 1e6 packets each in one batch (independent streams per
    simulation) against 16 reference batches of 1e6; the 30 radial bins
    within the gate and the total within 0.5 %."""
    from pyxopto_gb300.batched import BatchedMc
    from pyxopto_gb300.mcbase.mcutil import Axis
    n = 1_000_000
    ref = reference_batches('c4_semiinf_radial', BATCHES * n, ['top'])['top']
    layer = scenarios.BENCH['c4_semiinf_radial']['layers'][1]
    sims = {'mua': np.full(BATCHES, layer['mua']), 'mus': np.full(BATCHES, layer['mus']),
            'g': np.full(BATCHES, layer['pf'][1]), 'n': np.full(BATCHES, layer['n']),
            'num_packets': np.full(BATCHES, n, dtype=np.uint64)}
    b = BatchedMc(sims, raxis=Axis(0.0, 3e-3, 30), fast=True, seed=5)
    gpu = _stats.per_packet(b.run_raw(), n)
    _assert_gate(gpu, ref, 'batched radial bins')
    assert abs(gpu.sum(1).mean() / ref.sum(1).mean() - 1.0) < 5e-3
