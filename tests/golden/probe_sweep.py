"""The reference's linear fibre-probe validation tests
(xopto/mcml/test/validate.py:1227-1758: SingleLayerSixLinearProbe,
SingleLayerNineLinearProbe, SingleLayerGkLutSixLinearProbe): a uniform fibre
source in the first fibre of a six- or nine-fibre linear probe face
(LinearArray surface layout with a cutout and a reflective metal face) on
an 8 mm layer, the reflectance collected by the other fibres of a matching
LinearArray detector, for every point of an (mua, mus') sweep (and a
Gegenbauer gamma sweep).  The fixtures linear_probe_*.npz hold the
reference's values; its pass criterion is |mean relative error| < 0.5 %.
"""
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KEYS = ('hg_six', 'hg_nine', 'gk_six')


def load(key):
    return np.load(os.path.join(HERE, 'linear_probe_{}.npz'.format(key)))


def build(data, fast=True, scheduling='dynamic', rnginit=1):
    from pyxopto_gb300.mcml import mc
    from pyxopto_gb300.mcml.mcutil import fiber

    def pf(i):
        p = data['pf'][i]
        return mc.mcpf.Hg(float(p[0])) if int(data['pf_type'][0]) == 0 else mc.mcpf.Gk(float(p[0]), float(p[1]))

    def mmf(a):
        return fiber.MultimodeFiber(float(a[0]), float(a[1]), float(a[2]), float(a[3]))

    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=float(data['d'][i]), n=float(data['n'][i]), mua=0.0, mus=0.0, pf=pf(i))
        for i in range(3)])
    source = mc.mcsource.UniformFiber(mmf(data['source_fiber']),
                                      position=tuple(float(v) for v in data['source_position']))
    n, spacing, cw, ch, cn, diameter, refl = (float(v) for v in data['surface'])
    surface = mc.mcsurface.SurfaceLayouts(top=mc.mcsurface.LinearArray(
        mmf(data['surface_fiber']), n=int(n), spacing=spacing, cutout=(cw, ch), cutoutn=cn,
        diameter=diameter, reflectivity=refl))
    dn, dspacing = data['detector']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.LinearArray(
        mmf(data['detector_fiber']), n=int(dn), spacing=float(dspacing)))
    opts = [mc.mcoptions.McScheduling(scheduling)]
    if fast:
        opts.append(mc.mcoptions.McUseNativeMath(True))
    sim = mc.Mc(layers, source, det, surface=surface, options=opts, rnginit=rnginit)
    sim.rmax = float(data['rmax'][0])
    return sim


def grid(data):
    """(mua, mus', Gegenbauer g, Gegenbauer a) of every sweep point, in the
    order of the reference's loop (meshgrid 'ij')."""
    if 'gamma' in data.files:
        mua, musr, k = np.meshgrid(data['mua'], data['musr'], np.arange(data['gamma'].size), indexing='ij')
        return mua.ravel(), musr.ravel(), data['gk_g'][k.ravel()], data['gk_a'][k.ravel()]
    mua, musr = np.meshgrid(data['mua'], data['musr'], indexing='ij')
    return mua.ravel(), musr.ravel(), None, None


def run(sim, data, nphotons, stride=1):
    """Runs the sweep point by point (every ``stride``-th point); returns
    (reflectance of fibres 1.., reference values, seconds in Mc.run)."""
    mua, musr, gk_g, gk_a = grid(data)
    g = float(data['g'][0]) if 'g' in data.files else float(data['pf'][1][0])
    ref = data['reflectance'].reshape(mua.size, -1)
    out, t = [], 0.0
    idx = np.arange(0, mua.size, stride)
    for i in idx:
        sim.layers[1].mua = float(mua[i])
        sim.layers[1].mus = float(musr[i]) / (1.0 - g)
        if gk_g is not None:
            sim.layers[1].pf.g = float(gk_g[i])
            sim.layers[1].pf.a = float(gk_a[i])
        t0 = time.perf_counter()
        _, _, det = sim.run(nphotons)
        t += time.perf_counter() - t0
        out.append(det.top.reflectance[1:])
    return np.asarray(out), ref[idx], t


def relative_error(refl, ref):
    """Relative error (%) against the reference's values."""
    return (refl - ref) / ref * 100.0
