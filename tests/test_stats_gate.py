"""The statistical gate of the parity tests (tests/_stats.py) on synthetic
batches: it passes equal means, with independent and with strongly
correlated bins, at about its design rate, and it fails a shift of one
standard error in every bin."""
import numpy as np

import _stats


def _trials(make, n=60):
    rng = np.random.default_rng(7)
    fails = 0
    for t in range(n):
        a, b = make(rng)
        ok, _ = _stats.gate(a, b, draws=4000, seed=t)
        fails += not ok
    return fails


def test_gate_passes_independent_bins():
    assert _trials(lambda r: (r.normal(1.0, 0.1, (16, 100)), r.normal(1.0, 0.3, (16, 100)))) <= 1


def test_gate_passes_correlated_bins():
    def make(r):
        fa, fb = r.normal(0, 1, (16, 1)), r.normal(0, 1, (16, 1))
        a = 1 + 0.1 * (0.95 * fa + 0.31 * r.normal(0, 1, (16, 200)))
        b = 1 + 0.3 * (0.95 * fb + 0.31 * r.normal(0, 1, (16, 200)))
        return a, b
    assert _trials(make) <= 1


def test_gate_fails_a_one_sigma_shift():
    rng = np.random.default_rng(3)
    a = rng.normal(1.0, 0.1, (16, 100))
    b = rng.normal(1.0, 0.3, (16, 100))
    se = np.sqrt(0.1 ** 2 / 16 + 0.3 ** 2 / 16)
    ok, rep = _stats.gate(a, b + se)
    assert not ok, rep


def test_gate_constant_bins_must_agree():
    a = np.ones((16, 3))
    b = np.ones((16, 3))
    b[:, 1] = 2.0
    ok, rep = _stats.gate(a, b)
    assert not ok and rep['constant_bins_differing'] == 1
