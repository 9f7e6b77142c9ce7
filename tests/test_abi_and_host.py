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
    assert lib.mcgb_abi_version() == 1


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
