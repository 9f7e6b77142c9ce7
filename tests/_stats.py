"""Statistical gate shared by the parity tests that compare two Monte Carlo
estimates (FAST math against EXACT math, the GPU against the reference CPU
build).

Each side is given as independent batches: an array (K, bins) of per-batch
tallies normalised per packet.  Per bin, the difference of the batch means
over its standard error (Welch) is a t statistic, mapped to the normal
quantile of the same tail probability (z).  The gate is the north-star
criterion "within 3 sigma of the per-bin Monte Carlo error", made a test:

  * the number of bins with |z| > 3 must not exceed what chance gives, and
  * the sum of z^2 must be consistent with chance,

each with a tail probability above ``alpha`` (1e-3).  For independent bins
chance is the binomial share 2*(1 - Phi(3)) = 0.27 % of the bins and the
chi-square distribution.  Fluence voxels and depth slices are not
independent (one packet deposits into many of them), so the null
distributions of both statistics are taken from the batches themselves: the
difference of the means is redrawn as Gaussian combinations of each side's
centred batch deviations, which carry the measured covariance between bins.
With 16 batches and hundreds of bins the sample correlations are mostly
noise, so the measured correlation matrix is shrunk towards independence by
the share of its off-diagonal mass that the noise floor explains (the floor
is the same mass after the batches are shuffled bin by bin); for independent
bins this reproduces the binomial and chi-square answers.  Bins with no
variance on either side must agree exactly.
"""
import numpy as np
from scipy import stats

P3 = 2.0 * stats.norm.sf(3.0)


def z_scores(a, b):
    """(z over the bins with variance, mask of those bins, bins without
    variance that differ)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ka, kb = len(a), len(b)
    va = a.var(0, ddof=1) / ka
    vb = b.var(0, ddof=1) / kb
    se2 = va + vb
    ok = se2 > 0
    diff = a.mean(0) - b.mean(0)
    t = diff[ok] / np.sqrt(se2[ok])
    dof = se2[ok] ** 2 / (va[ok] ** 2 / (ka - 1) + vb[ok] ** 2 / (kb - 1))
    p = stats.t.sf(np.abs(t), dof)
    z = np.sign(t) * stats.norm.isf(np.maximum(p, 1e-300))
    bad_const = int(np.count_nonzero(diff[~ok] != 0.0))
    return z, ok, bad_const


def _offdiag_mass(da, db):
    """Sum of the squared off-diagonal entries of da^T da + db^T db."""
    ga, gb, gab = da @ da.T, db @ db.T, da @ db.T
    total = np.sum(ga ** 2) + np.sum(gb ** 2) + 2.0 * np.sum(gab ** 2)
    diag = np.sum((np.sum(da ** 2, 0) + np.sum(db ** 2, 0)) ** 2)
    return total - diag


def _shrinkage(da, db, rng, shuffles=4):
    """Weight of the independent part: noise-floor mass over measured mass."""
    mass = _offdiag_mass(da, db)
    if mass <= 0:
        return 1.0
    floor = 0.0
    for _ in range(shuffles):
        pa = np.take_along_axis(da, rng.permuted(np.tile(np.arange(len(da))[:, None], (1, da.shape[1])), axis=0), 0)
        pb = np.take_along_axis(db, rng.permuted(np.tile(np.arange(len(db))[:, None], (1, db.shape[1])), axis=0), 0)
        floor += _offdiag_mass(pa, pb) / shuffles
    return float(min(1.0, floor / mass))


def gate(a, b, alpha=1e-3, draws=20000, seed=12345):
    """Returns (passed, report) for the two batch arrays a and b."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    z, ok, bad_const = z_scores(a, b)
    n = int(z.size)
    count = int(np.count_nonzero(np.abs(z) > 3.0))
    chi2 = float(np.sum(z ** 2))
    # null distribution under the batch covariance
    se = np.sqrt(a[:, ok].var(0, ddof=1) / len(a) + b[:, ok].var(0, ddof=1) / len(b))
    da = (a[:, ok] - a[:, ok].mean(0)) / np.sqrt((len(a) - 1) * len(a)) / se
    db = (b[:, ok] - b[:, ok].mean(0)) / np.sqrt((len(b) - 1) * len(b)) / se
    rng = np.random.default_rng(seed)
    lam = _shrinkage(da, db, rng) if n > 1 else 1.0
    cnt_null = np.empty(draws, np.int64)
    chi_null = np.empty(draws, np.float64)
    step = 2000
    for s in range(0, draws, step):
        m = min(step, draws - s)
        zs = np.sqrt(1.0 - lam) * (rng.standard_normal((m, len(a))) @ da +
                                   rng.standard_normal((m, len(b))) @ db) + \
            np.sqrt(lam) * rng.standard_normal((m, n))
        cnt_null[s:s + m] = np.count_nonzero(np.abs(zs) > 3.0, axis=1)
        chi_null[s:s + m] = np.sum(zs ** 2, axis=1)
    p_count = float((np.count_nonzero(cnt_null >= count) + 1) / (draws + 1))
    p_chi2 = float((np.count_nonzero(chi_null >= chi2) + 1) / (draws + 1))
    report = {'bins': n, 'over_3sigma': count, 'expected_over_3sigma_independent': n * P3,
              'binomial_p': float(stats.binom.sf(count - 1, n, P3)) if n else 1.0,
              'chi2': chi2, 'chi2_independent_p': float(stats.chi2.sf(chi2, n)) if n else 1.0,
              'p_count': p_count, 'p_chi2': p_chi2, 'max_abs_z': float(np.max(np.abs(z))) if n else 0.0,
              'constant_bins_differing': bad_const, 'independent_share': lam}
    passed = bad_const == 0 and p_count > alpha and p_chi2 > alpha
    return passed, report


def record(what, report):
    """Appends a gate report to the JSON-lines file named by the environment
    variable MCGB_GATE_REPORT, when it is set (the numbers behind a passing
    test)."""
    import json
    import os
    path = os.environ.get('MCGB_GATE_REPORT')
    if path:
        test = os.environ.get('PYTEST_CURRENT_TEST', '').split(' ')[0]
        with open(path, 'a') as f:
            f.write(json.dumps(dict(report, test=test, what=what), default=float) + '\n')


def per_packet(rows, packets, k=8388607.0):
    """Integer tallies of batches -> per-packet weights (float64)."""
    return np.asarray(rows, np.float64) / k / float(packets)
