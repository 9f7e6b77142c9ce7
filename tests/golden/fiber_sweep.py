"""The reference's fibre validation and performance workload
(xopto/mcml/test/validate.py:348-511, SingleLayerUniformFiberRadial, timed by
test/performance.py): a normally incident multimode fibre (UniformFiberNI)
on an 8 mm layer between a fused-silica half-space and a water-like
half-space, a radial detector with the fibre's acceptance angle and rmax
5 mm, run once for each point of a 20 x 20 (mua, mus') grid; the radial
profiles are integrated over 200 um fibres at 5 source-detector separations
and compared with the CUDA-MCML values in cuda_mcml_fiber.npz.  The pass
criterion of the reference is |mean relative error| < 0.5 %.
"""
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(double=False):
    """The single-layer golden, or the two-layer one (validate.py:692-866:
    layer 1 fixed, the sweep on layer 2)."""
    return np.load(os.path.join(HERE, 'cuda_mcml_fiber2.npz' if double else 'cuda_mcml_fiber.npz'))


def build(data, fast=True, scheduling='dynamic', rnginit=1):
    from pyxopto_gb300.mcml import mc
    from pyxopto_gb300.mcml.mcutil import fiber
    g = data['g']
    layers = mc.mclayer.Layers([
        mc.mclayer.Layer(d=float(data['d'][i]), n=float(data['n'][i]), mua=0.0, mus=0.0,
                         pf=mc.mcpf.Hg(float(g[i]))) for i in range(len(g))])
    if 'fixed_layer' in data.files:
        k = int(data['fixed_layer'][0])
        layers[k].mua = float(data['fixed_mua'][0])
        layers[k].mus = float(data['fixed_musr'][0]) / (1.0 - float(g[k]))
    dcore, dclad, ncore, na = (float(v) for v in data['fiber'])
    source = mc.mcsource.UniformFiberNI(fiber.MultimodeFiber(dcore, dclad, ncore, na))
    start, stop, n = data['axis']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(
        mc.mcdetector.RadialAxis(float(start), float(stop), int(n)), cosmin=float(data['cosmin'][0])))
    opts = [mc.mcoptions.McScheduling(scheduling)]
    if fast:
        opts.append(mc.mcoptions.McUseNativeMath(True))
    sim = mc.Mc(layers, source, det, options=opts, rnginit=rnginit)
    sim.rmax = float(data['rmax'][0])
    return sim


def build_cartesian(data, fast=True, scheduling='dynamic', rnginit=1):
    """SingleLayerUniformFiberCartesian (xopto/mcml/test/validate.py:514-690):
    the same sample and source with a Cartesian detector of 1.1 x rmax by
    1.05 x rmax half-widths at the radial step, resampled to the radial axis
    by Cartesian.radial before the fibre integration.  Returns (simulator,
    radial axis)."""
    import numpy as np
    sim = build(data, fast=fast, scheduling=scheduling, rnginit=rnginit)
    from pyxopto_gb300.mcml import mc
    start, stop, nr = (float(v) for v in data['axis'])
    dr = stop / nr
    nx = np.ceil(nr * 2.2 / 2.0) * 2.0
    ny = np.ceil(nr * 2.1 / 2.0) * 2.0
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Cartesian(
        mc.mcdetector.Axis(-dr * nx * 0.5, dr * nx * 0.5, int(nx)),
        mc.mcdetector.Axis(-dr * ny * 0.5, dr * ny * 0.5, int(ny)), cosmin=float(data['cosmin'][0])))
    opts = [mc.mcoptions.McScheduling(scheduling)]
    if fast:
        opts.append(mc.mcoptions.McUseNativeMath(True))
    cart = mc.Mc(sim.layers, sim.source, det, options=opts, rnginit=rnginit)
    cart.rmax = sim.rmax
    return cart, mc.mcdetector.RadialAxis(start, stop, int(nr))


def build_vox(data, fast=True, scheduling='dynamic', rnginit=1):
    """The voxelized-medium version of the test (xopto/mcvox/test/validate.py:
    357-536): one voxel spanning +-2 rmax laterally and the layer thickness
    in depth, material 1 = the layer, material 0 = the fibre-side medium
    (also below the sample), the tilted-fibre source at normal incidence."""
    from pyxopto_gb300.mcvox import mc
    from pyxopto_gb300.mcvox.mcutil import fiber
    g = data['g']
    rmax = float(data['rmax'][0])
    A = mc.mcgeometry.Axis
    double = 'fixed_layer' in data.files
    if double:
        # DoubleLayerUniformFiberRadial (xopto/mcvox/test/validate.py:730-925):
        # 0.1 mm voxels in depth, material 1 down to the first layer's depth
        thickness = float(data['d'][1] + data['d'][2])
        zaxis = A(0.0, thickness, int(round(thickness / 0.1e-3)))
    else:
        zaxis = A(0.0, float(data['d'][1]), 1)
    voxels = mc.mcgeometry.Voxels(A(-2.0 * rmax, 2.0 * rmax, 1), A(-2.0 * rmax, 2.0 * rmax, 1), zaxis)
    materials = [mc.mcmaterial.Material(n=float(data['n'][i]), mua=0.0, mus=0.0, pf=mc.mcpf.Hg(float(g[i])))
                 for i in range(3 if double else 2)]
    if double:
        k = int(data['fixed_layer'][0])
        materials[k].mua = float(data['fixed_mua'][0])
        materials[k].mus = float(data['fixed_musr'][0]) / (1.0 - float(g[k]))
    dcore, dclad, ncore, na = (float(v) for v in data['fiber'])
    source = mc.mcsource.UniformFiber(fiber.MultimodeFiber(dcore, dclad, ncore, na))
    start, stop, n = data['axis']
    det = mc.mcdetector.Detectors(top=mc.mcdetector.Radial(
        mc.mcdetector.RadialAxis(float(start), float(stop), int(n)), cosmin=float(data['cosmin'][0])))
    opts = [mc.mcoptions.McScheduling(scheduling)]
    if fast:
        opts.append(mc.mcoptions.McUseNativeMath(True))
    sim = mc.Mc(voxels, materials, source, det, options=opts, rnginit=rnginit)
    sim.rmax = rmax
    sim.voxels.material[...] = 1
    if double:
        zc = zaxis.centers
        sim.voxels.material[zc > float(data['d'][1]), :, :] = 2
    return sim


def run(sim, data, nphotons, raxis=None):
    """Runs the 400 simulations in sequence (as the reference does); returns
    (fibre reflectance [20, 20, 5], seconds spent in Mc.run)."""
    from pyxopto_gb300.util import convolve
    mua, musr = np.meshgrid(data['mua'], data['musr'], indexing='ij')
    k = int(data['sweep_layer'][0]) if 'sweep_layer' in data.files else 1
    g = float(data['g'][k])
    profiles, r = [], None
    t = 0.0
    target = sim.materials[k] if hasattr(sim, 'materials') else None
    for i in range(mua.size):
        obj = target if target is not None else sim.layers[k]
        obj.mua = float(mua.flat[i])
        obj.mus = float(musr.flat[i]) / (1.0 - g)
        t0 = time.perf_counter()
        _, _, det = sim.run(nphotons)
        t += time.perf_counter() - t0
        if raxis is not None:
            profiles.append(det.top.radial(raxis).reflectance)
            r = raxis.centers
        else:
            profiles.append(det.top.reflectance)
            r = det.top.r
    refl = convolve.fiber_reflectance(r, np.asarray(profiles), sds=list(data['sds']),
                                      dcore=float(data['sds_dcore'][0]))
    return refl.reshape(data['reflectance'].shape), t


def relative_error(data, refl):
    """Relative error (%) against the CUDA-MCML values."""
    return (refl - data['reflectance']) / data['reflectance'] * 100.0
