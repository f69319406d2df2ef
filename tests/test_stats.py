"""The blocking analysis that attaches error bars to the shift and projected energy, against
the reference's own tests of it (test/StatsTools.jl:33-62).  CPU only."""
import math
import warnings

import numpy as np
import pytest

from rimugpu.stats import blocking_analysis


def smoothen(x, b):
    """Periodic moving average over b points, centred as the reference's smoothen
    (src/StatsTools/growth_witness.jl:66-77): point i averages x[i - b//2 .. i - b//2 + b - 1]."""
    off = b // 2
    return sum(np.roll(x, -d) for d in range(-off, b - off)) / b


@pytest.mark.parametrize("seed", range(4))
def test_independent_and_correlated_series(seed):
    """2^10 independent normal samples need no blocking (k <= 4) and give an error between
    0.01 and 0.04; smoothing over 2^5 points correlates them, so the M-test picks a level with
    5 < k <= 7, with the same mean and an error in the same range."""
    v = np.random.default_rng(seed).normal(size=2 ** 10)
    br = blocking_analysis(v)
    assert 0.01 < br.err < 0.04 and br.k <= 4
    brs = blocking_analysis(smoothen(v, 2 ** 5))
    assert br.mean == pytest.approx(v.mean()) and brs.mean == pytest.approx(v.mean())
    assert 0.01 < brs.err < 0.04 and 5 < brs.k <= 7


def test_blocking_fails_on_series_without_information():
    """A constant series fails the M-test (k = -1, NaN error, with a warning), and so do a
    single point and an empty series."""
    for x in (np.ones(2000), np.array([1.0]), np.array([])):
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("always")
            r = blocking_analysis(x)
        assert r.k == -1 and math.isnan(r.err), len(x)
        assert caught, len(x)


@pytest.mark.parametrize("seed", range(4))
def test_ratio_of_means_against_linear_error_propagation(seed):
    """The projected-energy estimator on the reference's well-behaved example
    (test/StatsTools.jl:131-155): 2 000 samples of a bivariate normal with means 2 and 3,
    standard errors of the means 0.5 and 0.1 and their covariance 0.02.  The ratio lies within
    2 sigma_f of 2/3 and the error agrees with linear error propagation (x_by_y_linear,
    ratio_of_means.jl:166-171) to 8/sqrt(n); after correlating the series by smoothing over
    2^3 and 2^6 points the blocked ratio and error stay within 2 sigma_f."""
    from rimugpu.stats import ratio_of_means
    n, ma, mb, sa, sb, rho = 2000, 2.0, 3.0, 0.5, 0.1, 0.02
    f = ma / mb
    sf = math.sqrt((sa / mb) ** 2 + (ma * sb / mb ** 2) ** 2 - 2 * rho * ma / mb ** 3)
    cov = np.array([[sa ** 2, rho], [rho, sb ** 2]]) * n
    ab = np.random.default_rng(seed).multivariate_normal([ma, mb], cov, size=n)
    a, b = ab[:, 0], ab[:, 1]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        r, err = ratio_of_means(a, b)
        rs, errs = ratio_of_means(smoothen(a, 2 ** 3), smoothen(b, 2 ** 6))
    assert abs(r - f) <= 2 * sf
    assert err == pytest.approx(sf, rel=8 / math.sqrt(n))
    assert abs(rs - f) <= 2 * sf and abs(errs - sf) <= 2 * sf


def test_ratio_of_means_without_variance():
    """Zero-variance examples of test/StatsTools.jl:105-109: value and error are 0 for a zero
    numerator, and the ratio of two constant series is exact."""
    from rimugpu.stats import ratio_of_means
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert ratio_of_means([0, 0, 0, 0, 0, 0], [1, 1, 1, 1, 1, 2]) == (0.0, 0.0)
        assert ratio_of_means(np.ones(2000), np.ones(2000)) == (1.0, 0.0)
