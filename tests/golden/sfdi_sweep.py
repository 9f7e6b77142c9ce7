"""The reference's SFDI validation test (xopto/mcml/test/validate.py:867-1050,
SingleLayerSfdiIncidence30VariableNa): a Line source at 30 degrees incidence
on a semi-infinite layer (n 1.46, mua 110 1/m, mus 4333 1/m, HG 0.7), a
SymmetricX detector on a 4000-point log axis to 150 mm, one run per detector
NA; the profile is transformed to spatial frequencies 0-1000 1/m
(discreteSimpson) and its amplitude and phase are compared with the values in
sfdi_30deg_variable_na.npz.  The reference passes when, for NA indices 4..,
the largest per-NA mean |relative amplitude error| is below 2.5 % and the
largest mean |phase error| below 0.025 rad.
"""
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    return np.load(os.path.join(HERE, 'sfdi_30deg_variable_na.npz'))


def run(data, nphotons, na_indices, fast=True, scheduling='dynamic', rnginit=1):
    """Amplitude and phase [len(na_indices), frequencies] and the seconds
    spent in Mc.run."""
    from pyxopto_gb300.mcml import mc
    from pyxopto_gb300.mcml.mcutil import fourier
    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=float(data['d'][i]), n=float(data['n'][i]), mua=float(data['mua'][i]),
                         mus=float(data['mus'][i]), pf=mc.mcpf.Hg(float(data['g'][i])))
        for i in range(3)])
    source = mc.mcsource.Line(direction=tuple(float(v) for v in data['direction']))
    center, rng, n_half, logscale = data['axis']
    opts = [mc.mcoptions.McScheduling(scheduling)]
    if fast:
        opts.append(mc.mcoptions.McUseNativeMath(True))
    out = np.zeros((len(na_indices), data['frequencies'].size), dtype=np.complex128)
    t = 0.0
    for k, i in enumerate(na_indices):
        cosmin = float(np.sqrt(1.0 - data['na'][i] ** 2))
        det = mc.mcdetector.Detectors(top=mc.mcdetector.SymmetricX(
            mc.mcdetector.SymmetricAxis(float(center), float(rng), int(n_half), logscale=bool(logscale)),
            cosmin=cosmin))
        sim = mc.Mc(layers, source, det, options=opts, rnginit=rnginit + k)
        sim.rmax = float(data['rmax'][0])
        t0 = time.perf_counter()
        _, _, res = sim.run(nphotons)
        t += time.perf_counter() - t0
        out[k] = fourier.discreteSimpson(data['frequencies'], res.top.x, res.top.reflectance, uneven=True)
    return np.abs(out), np.angle(out), t


def errors(data, na_indices, amplitude, phase):
    """Per-NA mean |relative amplitude error| and mean |phase error| (rad)."""
    ref_a = data['amplitude'][na_indices]
    ref_p = data['phase'][na_indices]
    return (np.mean(np.abs((amplitude - ref_a) / ref_a), 1), np.mean(np.abs(phase - ref_p), 1))
