"""The k = exp(g) coefficient field of the learned-smoother workload: g has the requested
standard deviation, and its empirical autocorrelation follows the squared-exponential
covariance exp(-r^2 / (2 ell^2)) of correlation length ell (in macro elements)."""

import numpy as np

from sfem_gb300.coefficients import gaussian_random_field, lognormal_coefficient


def _corr(g, lag, axis):
    a = np.take(g, range(0, g.shape[axis] - lag), axis=axis)
    b = np.take(g, range(lag, g.shape[axis]), axis=axis)
    return float(np.mean(a * b) / np.mean(g * g))


def test_sigma_and_mean():
    for seed in range(3):
        g = gaussian_random_field((32, 32, 32), ell=8.0, sigma=1.0, seed=seed)
        assert abs(g.std() - 1.0) < 1e-12 and abs(g.mean()) < 1e-12
        k = lognormal_coefficient(32, 32, 32, ell=8.0, sigma=1.0, seed=seed)
        assert k.dtype == np.float32 and k.size == 32 ** 3 and (k > 0).all()
        assert abs(np.log(k.astype(np.float64)).std() - 1.0) < 1e-6


def test_correlation_length():
    # a domain of 12 correlation lengths keeps the bias of the sample normalisation small
    ell = 8.0
    lags = (2, 4, 8)
    est = {l: [] for l in lags}
    for seed in range(4):
        g = gaussian_random_field((96, 96, 96), ell=ell, sigma=1.0, seed=seed)
        for l in lags:
            est[l].append(np.mean([_corr(g, l, ax) for ax in range(3)]))
    for l in lags:
        expect = np.exp(-l * l / (2 * ell * ell))
        assert abs(np.mean(est[l]) - expect) < (0.02 if l < 8 else 0.04), (l, np.mean(est[l]), expect)
    # a shorter correlation length decorrelates faster
    g2 = gaussian_random_field((96, 96, 96), ell=2.0, sigma=1.0, seed=0)
    assert np.mean([_corr(g2, 4, ax) for ax in range(3)]) < 0.25
