"""The surrogate's Monte Carlo judge: the two-halves estimator removes the
judge's own Monte Carlo noise from the measured error (CPU, synthetic
profiles with a planted error and planted noise)."""
import numpy as np

from pyxopto_gb300.surrogate import Surrogate


def _profiles(rng, n=4000, bins=30):
    return np.exp(-np.linspace(0.0, 4.0, bins))[None, :] * rng.uniform(0.5, 2.0, (n, 1))


def test_judge_removes_mc_noise():
    rng = np.random.default_rng(3)
    truth = _profiles(rng)
    pred = truth * (1.0 + 0.008 * rng.standard_normal(truth.shape))      # 0.8 % planted error
    sig = 0.009 * np.sqrt(2.0)                                            # each half: 1.27 %
    a = truth * (1.0 + sig * rng.standard_normal(truth.shape))
    b = truth * (1.0 + sig * rng.standard_normal(truth.shape))
    err, raw, noise = Surrogate.judge_error(pred, a, b)
    assert abs(np.sqrt(np.mean(noise ** 2)) - 0.009) < 0.0005
    assert np.sqrt(np.mean(raw ** 2)) > 0.0115                               # noise inflates it
    assert abs(np.sqrt(np.mean(err ** 2)) - 0.008) < 0.0006                  # corrected


def test_judge_exact_prediction_scores_near_zero():
    rng = np.random.default_rng(4)
    truth = _profiles(rng, n=2000)
    a = truth * (1.0 + 0.02 * rng.standard_normal(truth.shape))
    b = truth * (1.0 + 0.02 * rng.standard_normal(truth.shape))
    err, raw, _ = Surrogate.judge_error(truth.copy(), a, b)
    # the per-profile estimate is clipped at zero; its median is zero and
    # its mean square a small fraction of the uncorrected one
    assert np.median(err) == 0.0
    assert np.mean(err ** 2) < 0.2 * np.mean(raw ** 2)


def test_judge_mask_ignores_empty_bins():
    truth = np.ones((3, 30))
    truth[:, 20:] = 0.0
    a = truth.copy()
    b = truth.copy()
    pred = truth.copy()
    pred[:, 20:] = 5.0                      # masked bins may be anything
    err, _, _ = Surrogate.judge_error(pred, a, b, mask=truth > 0)
    assert np.all(err == 0.0)
