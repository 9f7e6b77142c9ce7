"""C ABI surface and host-side logic that needs no GPU: every symbol that
include/xopto_gb300.h declares is exported, struct layouts agree, and the
library rejects invalid configurations before launching anything."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, 'include'))):
        if fn.endswith('.h'):
            text = open(os.path.join(ROOT, 'include', fn)).read()
            names += re.findall(r'^\s*(?:const\s+)?\w+\s*\*?\s*(mcgb_\w+)\s*\(', text, re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts(lib):
    from pyxopto_gb300 import _abi
    _abi.check_layout(lib.mcgb_sizeof)
    assert lib.mcgb_sizeof(0) == 72 and lib.mcgb_sizeof(5) == 64 and lib.mcgb_sizeof(99) == -1
    assert lib.mcgb_abi_version() == 3


def _valid_cfg():
    import scenarios
    mc = scenarios.build_mc('c1_line_hg_radial')
    cfg = mc.pack(1000, 8)
    from pyxopto_gb300 import _abi
    b = _abi.McgbBuffers()
    b.rng_x, b.rng_a, b.counters = 16, 16, 16          # never dereferenced: checks fail first
    b.accumulator, b.accumulator_size = 16, mc._acc.size
    return mc, cfg, b


def _run(lib, cfg, b):
    from pyxopto_gb300 import _abi
    return lib.mcgb_mcml_run(C.byref(cfg), C.byref(b), None)


def test_validation_rejects_bad_configs(lib):
    from pyxopto_gb300 import _abi
    mc, cfg, b = _valid_cfg()
    cfg.num_layers = 2
    assert _run(lib, cfg, b) == _abi.E_INVALID
    assert b'num_layers' in lib.mcgb_last_error()
    mc, cfg, b = _valid_cfg()
    cfg.top.offset = b.accumulator_size          # radial bins beyond the buffer
    assert _run(lib, cfg, b) == _abi.E_SIZE
    mc, cfg, b = _valid_cfg()
    cfg.opt.method = 7
    assert _run(lib, cfg, b) == _abi.E_INVALID
    mc, cfg, b = _valid_cfg()
    b.rng_x = None
    assert _run(lib, cfg, b) == _abi.E_INVALID
    mc, cfg, b = _valid_cfg()
    cfg.num_streams = 0
    assert _run(lib, cfg, b) == _abi.E_INVALID
    mc, cfg, b = _valid_cfg()
    cfg.pf_kind = _abi.PF_LUT                    # LUT phase function without a table
    assert _run(lib, cfg, b) == _abi.E_INVALID
    mc, cfg, b = _valid_cfg()
    cfg.trace.flags = _abi.TRACE_ALL
    cfg.trace.max_events = 4
    assert _run(lib, cfg, b) == _abi.E_SIZE     # no trace buffers


def test_mlp_entry_points_validate_arguments(lib):
    """The surrogate's GEMM-path switch and multi-tensor AdamW reject bad
    arguments before touching the device; scratch sizes follow the row
    chunking."""
    from pyxopto_gb300 import _abi
    assert lib.mcgb_mlp_gemm_path(-1) in (0, 1)
    assert lib.mcgb_mlp_gemm_path(5) == -1
    assert b'GEMM path' in lib.mcgb_last_error()
    tab = (_abi.McgbAdamwTensor * (_abi.ADAMW_MAX_TENSORS + 1))()
    for count in (0, _abi.ADAMW_MAX_TENSORS + 1):
        assert lib.mcgb_mlp_adamw_multi(tab, count, 1e-3, 0.9, 0.999, 1e-8, 1, None) == _abi.E_INVALID
    assert lib.mcgb_mlp_adamw_multi(tab, 1, 1e-3, 0.9, 0.999, 1e-8, 1, None) == _abi.E_INVALID
    assert b'tensor 0' in lib.mcgb_last_error()
    assert lib.mcgb_mlp_adamw_multi(tab, 1, 1e-3, 0.9, 0.999, 1e-8, 0, None) == _abi.E_INVALID
    assert lib.mcgb_mlp_act_bwd_scratch(4096, 256) == 64 * 256
    assert lib.mcgb_mlp_act_bwd_scratch(0, 256) == 0
    assert lib.mcgb_mlp_bwd_weight_scratch(0, 256, 256) == 0
    assert lib.mcgb_mlp_bwd_weight_scratch(4096, 256, 256) % (256 * 256) == 0


def test_zero_packets_is_a_no_op(lib):
    mc, cfg, b = _valid_cfg()
    cfg.num_packets = 0
    assert _run(lib, cfg, b) == 0


def test_reduce_tallies_exact(lib):
    from pyxopto_gb300 import parallel
    a = np.array([2 ** 63, 5, 2 ** 64 - 1], dtype=np.uint64)
    b = np.array([2 ** 63, 7, 1], dtype=np.uint64)
    out = parallel.host_reduce(a.copy(), b)
    assert out.tolist() == [0, 12, 0]            # modulo 2^64, like the device sums


def test_options_and_plugins():
    from pyxopto_gb300.mcml import mc
    from pyxopto_gb300.mcbase import mcoptions
    r = mcoptions.resolve([mc.mcoptions.McMethod('mbl'), mc.mcoptions.McUseNativeMath(True),
                           ('MC_PACKET_WEIGHT_MIN', 1e-3)])
    assert r['MC_METHOD'] == 2 and r['MC_USE_NATIVE_MATH'] and r['MC_PACKET_WEIGHT_MIN'] == 1e-3
    with pytest.raises(ValueError):
        mcoptions.resolve([mcoptions.McUseEnhancedRng(True)])
    ax = mc.mcdetector.RadialAxis(0.0, 1e-3, 4)
    e = ax.edges
    np.testing.assert_allclose(ax.centers, 2 / 3 * (e[:-1] ** 2 + e[:-1] * e[1:] + e[1:] ** 2) /
                               (e[:-1] + e[1:]))
    with pytest.raises(ValueError):
        mc.Mc(mc.mclayer.Layers([mc.mclayer.Layer(0, 1, 0, 0, mc.mcpf.Hg(0))] * 2), mc.mcsource.Line())
    # Fresnel closed form at normal incidence
    from pyxopto_gb300.mcbase import mcutil
    assert abs(mcutil.reflectance(1.0, 1.33) - (0.33 / 2.33) ** 2) < 1e-15


def test_sampling_volume_validation(lib):
    """mcgb_sampling_volume checks the grid, the accumulator range and the
    trace size before it launches anything (no GPU needed)."""
    from pyxopto_gb300 import _abi
    from pyxopto_gb300.mcml import mcsv

    def cfg():
        sv = mcsv.SamplingVolume(mcsv.Axis(-1e-3, 1e-3, 4), mcsv.Axis(-1e-3, 1e-3, 5),
                                 mcsv.Axis(0.0, 1e-3, 3))
        c = sv.pack(None)
        c.max_events, c.num_packets = 10, 7
        return c

    def call(c, trace=16, floats=7 * 10 * 8, accu_size=60):
        return lib.mcgb_sampling_volume(C.byref(c), C.c_void_p(trace), floats, C.c_void_p(16),
                                        C.c_void_p(16), accu_size, C.c_void_p(16), None, None)

    assert lib.mcgb_sampling_volume(None, None, 0, None, None, 0, None, None, None) == _abi.E_INVALID
    c = cfg()
    c.shape[1] = 0
    assert call(c) == _abi.E_INVALID
    c = cfg()
    c.voxel_size[2] = 0.0
    assert call(c) == _abi.E_INVALID
    assert call(cfg(), accu_size=59) == _abi.E_SIZE
    c = cfg()
    c.offset = 1
    assert call(c) == _abi.E_SIZE
    assert call(cfg(), floats=7 * 10 * 8 - 1) == _abi.E_SIZE
    c = cfg()
    c.max_events = 0
    assert call(c) == _abi.E_INVALID
    assert call(cfg(), trace=8) == _abi.E_INVALID             # not 16-byte aligned
    assert b'aligned' in lib.mcgb_last_error()
    c = cfg()
    c.num_packets = 0
    assert call(c) == _abi.OK                                # nothing to do, no launch


def test_sampling_volume_host_objects():
    """SamplingVolume packing and scaling (xopto/mcbase/mcsv.py:313-395) and
    the trace maxlen rules (xopto/mcbase/mctrace.py:848-857)."""
    from pyxopto_gb300.mcml import mcsv, mctrace
    sv = mcsv.SamplingVolume(mcsv.Axis(-1e-3, 1e-3, 4), mcsv.Axis(-1e-3, 1e-3, 5),
                             mcsv.Axis(0.0, 1e-3, 2))
    c = sv.pack(None)
    assert list(c.shape) == [4, 5, 2] and c.k == 0x7FFFFF
    assert abs(c.multiplier - 1.0 / 4e-4) < 1e-3 and abs(c.top_left[0] + 1e-3) < 1e-9
    raw = np.arange(40, dtype=np.uint64)
    sv.update_data(None, [raw], total_weight=np.array([0x7FFFFF * 3], dtype=np.uint64))
    assert sv.data.shape == (2, 5, 4) and sv.weight == 3.0
    assert np.allclose(sv.data.ravel(), raw / (0x7FFFFF / 4e-4))
    sv.update_data(None, [raw], total_weight=np.array([0x7FFFFF], dtype=np.uint64))
    assert sv.weight == 4.0
    sv2 = mcsv.SamplingVolume.fromdict(sv.todict())
    assert sv2.shape == sv.shape and sv2.data is None
    assert mctrace.Trace(100, options=mctrace.Trace.TRACE_START).maxlen == 1
    assert mctrace.Trace(100, options=mctrace.Trace.TRACE_START | mctrace.Trace.TRACE_END).maxlen == 2
    assert mctrace.Trace(100).maxlen == 100
    with pytest.raises(TypeError):
        mctrace.Filter(x=0.5)


def test_reference_unbuildable_combinations_rejected(lib):
    """Combinations the reference does not offer are refused before any
    launch: a rectangular source with a specular detector (its launch code
    does not build, xopto/mcml/mcsource/rectangular.py:141) and the
    look-up-table detectors other than TotalLut in voxelized media
    (xopto/mcvox/mcdetector/__init__.py)."""
    import scenarios
    from pyxopto_gb300 import _abi
    spec = dict(scenarios.SCENARIOS['rect_uniform'])
    spec['detectors'] = dict(spec['detectors'], specular=dict(type='Total'))
    mc = scenarios.build_mc(spec)
    cfg = mc.pack(1000, 8)
    b = _abi.McgbBuffers()
    b.rng_x, b.rng_a, b.counters = 16, 16, 16
    b.accumulator, b.accumulator_size = 16, mc._acc.size
    assert lib.mcgb_mcml_run(C.byref(cfg), C.byref(b), None) == _abi.E_UNSUPPORTED
    assert b'specular' in lib.mcgb_last_error()
    vox = scenarios.build_mc('vox_cartesian')
    vcfg, _ = vox.pack(1000, 8)
    vcfg.top.kind = _abi.DET_FIBER_LUT_ARRAY
    vcfg.top.n, vcfg.top.n_y, vcfg.top.table_offset = 1, 16, 0
    vcfg.top.offset = 0
    vb = _abi.McgbBuffers()
    vb.rng_x, vb.rng_a, vb.counters, vb.voxels, vb.materials = 16, 16, 16, 16, 16
    vb.accumulator, vb.accumulator_size = 16, vox._acc.size
    vb.fp_lut, vb.fp_lut_size = 16, 16
    assert lib.mcgb_mcvox_run(C.byref(vcfg), C.byref(vb), None) == _abi.E_UNSUPPORTED
    assert b'TotalLut only' in lib.mcgb_last_error()


def test_sampling_volume_needs_a_trace():
    import scenarios
    from pyxopto_gb300.mcml import mcsv
    mc = scenarios.build_mc('c1_line_hg_radial')
    sv = mcsv.SamplingVolume(mcsv.Axis(0, 1e-3, 2), mcsv.Axis(0, 1e-3, 2), mcsv.Axis(0, 1e-3, 2))
    with pytest.raises(RuntimeError):
        mc.sampling_volume(None, sv)


def test_lut_classes():
    """LinearLut interpolation and the CDF inversion of EmissionLut
    (xopto/mcbase/mcutil/lut.py:155-325): an isotropic radiance over
    cos(theta) in [0, 1] has the density sin(theta), so the table is
    monotone and spans [0, 1]."""
    from pyxopto_gb300.mcml.mcutil import lut
    ll = lut.LinearLut([0.0, 1.0, 4.0], first=1.0, last=3.0)
    assert np.allclose(ll([1.0, 1.5, 2.0, 2.5, 3.0]), [0.0, 0.5, 1.0, 2.5, 4.0])
    em = lut.EmissionLut(np.ones(50), n=200)
    assert em.data.size == 200 and abs(em.data[0]) < 1e-9 and abs(em.data[-1] - 1.0) < 1e-9
    assert np.all(np.diff(em.data) >= 0.0)
    col = lut.CollectionLut([0.0, 1.0], costheta=[0.5, 1.0], n=11)
    assert col.first == 0.5 and col.last == 1.0 and np.allclose(col.data, np.linspace(0, 1, 11))


def test_cartesian_to_radial_conversion():
    """Cartesian.radial (xopto/mcml/mcdetector/cartesian.py:289-327): a
    uniform Cartesian reflectance stays the same reflectance on every ring
    that lies inside the grid."""
    from pyxopto_gb300.mcml import mcdetector
    cart = mcdetector.Cartesian(mcdetector.Axis(-1e-3, 1e-3, 40), mcdetector.Axis(-1e-3, 1e-3, 40))
    cart.set_raw_data(np.full(cart.shape, 3.0), 1000)
    rad = cart.radial(mcdetector.RadialAxis(0.0, 8e-4, 16))
    assert np.allclose(rad.reflectance, cart.reflectance[0, 0], rtol=1e-6)


def test_voxelized_surface_layouts_refused():
    """None of the reference's voxelized surface layouts builds into its
    kernel (xopto/mcvox/mcsurface), so mcvox.Mc takes only the default
    layouts and refuses the others with an explanation."""
    import scenarios
    from pyxopto_gb300.mcvox import mc
    m = scenarios.build_mc('vox_cartesian')
    mc.Mc(m.voxels, m.materials, m.source, surface=mc.mcsurface.SurfaceLayouts())
    with pytest.raises(ValueError, match='do not build'):
        mc.Mc(m.voxels, m.materials, m.source,
              surface=mc.mcsurface.SurfaceLayouts(bottom=mc.mcsurface.LambertianReflector(0.5)))


def test_run_helper_configuration():
    """McRunHelper builds its simulator from the create_* hooks in the
    reference's order and reports the configuration (mcrun/helper.py)."""
    from pyxopto_gb300.mcml import mcrun
    h = mcrun.McRunHelper()
    cfg = h.collect_mc_config()
    assert cfg['detectors'] is not None and cfg['fluence'] is None and cfg['trace'] is None
    assert h.collect_detectors(None) == {'reflectance': None, 'transmittance': None, 'specular': None}
