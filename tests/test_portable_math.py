"""Accuracy of the portable single-precision log/exp/sincos/powr/cbrt that the
EXACT math mode evaluates identically on the GPU and the CPU."""
import numpy as np


def ulp_err(got, want):
    got = np.asarray(got, dtype=np.float64)
    want32 = np.asarray(want, dtype=np.float32)
    ulp = np.spacing(np.abs(want32)).astype(np.float64)
    return np.abs(got - np.asarray(want, np.float64)) / ulp


def test_log(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(0)
    u = np.concatenate([rng.random(20000).astype(np.float32),
                        np.float32(2.0) ** rng.uniform(-140, 120, 5000).astype(np.float32),
                        np.array([1.0, 0.5, 2.0, 1e-38, 3e-45, 0.99999994], np.float32)])
    u = u[u > 0]
    got = np.array([lib.mco_pm_log(float(v)) for v in u])
    err = ulp_err(got, np.log(u.astype(np.float64)))
    # absolute accuracy near 1 where log -> 0
    close = np.abs(np.log(u.astype(np.float64))) < 1e-3
    assert np.max(err[~close]) <= 3.0
    assert np.max(np.abs(got[close] - np.log(u[close].astype(np.float64)))) < 2e-10
    assert np.isneginf(lib.mco_pm_log(0.0))
    assert np.isnan(lib.mco_pm_log(-1.0))


def test_exp(oracle):
    lib = oracle.load()
    x = np.linspace(-87, 88, 20011).astype(np.float32)
    got = np.array([lib.mco_pm_exp(float(v)) for v in x])
    assert np.max(ulp_err(got, np.exp(x.astype(np.float64)))) <= 3.0
    assert lib.mco_pm_exp(-200.0) == 0.0 and np.isinf(lib.mco_pm_exp(100.0))


def test_sincos(oracle):
    import ctypes as C
    lib = oracle.load()
    x = np.concatenate([np.linspace(0, 2 * np.pi, 20000), np.linspace(-20, 20, 2001)]).astype(np.float32)
    s, c = C.c_float(), C.c_float()
    gs, gc = [], []
    for v in x:
        lib.mco_pm_sincos(float(v), C.byref(s), C.byref(c))
        gs.append(s.value)
        gc.append(c.value)
    x64 = x.astype(np.float64)
    assert np.max(np.abs(np.array(gs) - np.sin(x64))) < 2.5e-7
    assert np.max(np.abs(np.array(gc) - np.cos(x64))) < 2.5e-7


def test_powr(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(1)
    x = rng.uniform(0.05, 4.0, 5000).astype(np.float32)
    y = rng.uniform(-3.0, 3.0, 5000).astype(np.float32)
    got = np.array([lib.mco_pm_pow(float(a), float(b)) for a, b in zip(x, y)])
    want = np.power(x.astype(np.float64), y.astype(np.float64))
    assert np.max(np.abs(got - want) / want) < 2e-6
    assert lib.mco_pm_pow(0.0, 2.0) == 0.0 and lib.mco_pm_pow(1.0, 7.0) == 1.0


def test_cbrt(oracle):
    """cbrt(2u - 1) of the MHg/MPc samplers: within 2 ulp on [-1, 1] and
    beyond, odd, and exact at 0, +-1 and +-8."""
    lib = oracle.load()
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-1.0, 1.0, 20000),
                        np.float32(2.0) ** rng.uniform(-120, 120, 4000)]).astype(np.float32)
    got = np.array([lib.mco_pm_cbrt(float(v)) for v in x])
    want = np.cbrt(x.astype(np.float64))
    assert np.max(ulp_err(got, want)) <= 2.0
    assert all(lib.mco_pm_cbrt(float(-v)) == -lib.mco_pm_cbrt(float(v)) for v in x[:200])
    for v in (0.0, 1.0, -1.0, 8.0, -8.0):
        assert lib.mco_pm_cbrt(v) == np.cbrt(v)


def test_analytic_pf_pack():
    """Hg2/MHg/Pc/MPc pack their parameters and sampler kind into McgbPf
    and round-trip through todict."""
    from pyxopto_gb300 import _abi
    from pyxopto_gb300.mcml import mcpf
    cases = [(mcpf.Hg2(0.9, -1.5, 0.25), _abi.PF_EXT_HG2, [0.9, -1.0, 0.25]),
             (mcpf.MHg(0.8, 0.6), _abi.PF_EXT_MHG, [0.8, 0.6]),
             (mcpf.Pc(12.0), _abi.PF_EXT_PC, [12.0]),
             (mcpf.MPc(20.0, 0.85), _abi.PF_EXT_MPC, [20.0, 0.85]),
             (mcpf.MGk(0.8, 0.0, 0.9), _abi.PF_EXT_MGK,
              [0.8, 0.9, 0.0, (1 + 0.64) / 1.6, (1 + 1.6 + 0.64) / 1.6])]
    for pf, ext, params in cases:
        t = pf.pack(None, _abi.McgbPf())
        assert pf.kind == _abi.PF_EXT and t.ext_kind == ext
        np.testing.assert_allclose(list(t.p)[:len(params)], params, rtol=1e-7)
        again = mcpf.pf_fromdict(pf.todict())
        assert type(again) is type(pf) and again.todict() == pf.todict()
