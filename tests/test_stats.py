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
    (test/StatsTools.jl:111-155): 2 000 samples of a bivariate normal with means 2 and 3,
    standard errors of the means 0.5 and 0.1 and their covariance 0.02.  The ratio and the
    Monte Carlo median lie within 2 sigma_f of 2/3; the linear error and the distances from the
    median to the 16 % and 84 % quantiles agree with linear error propagation (x_by_y_linear,
    ratio_of_means.jl:166-171) to 8/sqrt(n); after correlating the series by smoothing over
    2^3 and 2^6 points the M-test picks 6 <= k <= 8 and ratio, error and quantiles stay within
    2 sigma_f."""
    from rimugpu.stats import ratio_of_means, x_by_y_linear
    n, ma, mb, sa, sb, rho = 2000, 2.0, 3.0, 0.5, 0.1, 0.02
    f, sf = x_by_y_linear(ma, mb, sa, sb, rho)
    assert f == pytest.approx(ma / mb)
    # uncorrelated: the propagated error of Measurements.jl, sqrt((sa/mb)^2 + (ma sb/mb^2)^2)
    assert x_by_y_linear(ma, mb, sa, sb, 0)[1] == pytest.approx(math.hypot(sa / mb, ma * sb / mb ** 2))
    cov = np.array([[sa ** 2, rho], [rho, sb ** 2]]) * n
    ab = np.random.default_rng(seed).multivariate_normal([ma, mb], cov, size=n)
    a, b = ab[:, 0], ab[:, 1]
    r = ratio_of_means(a, b, warn=False, rng=seed)
    assert r.k <= 4 and r.success
    assert abs(r.f - f) <= 2 * sf and abs(r.pmedian() - f) <= 2 * sf
    q = r.pquantile([0.16, 0.5, 0.84])
    assert q[2] - q[1] == pytest.approx(sf, rel=8 / math.sqrt(n))
    assert q[1] - q[0] == pytest.approx(sf, rel=8 / math.sqrt(n))
    assert r.sigma_f == pytest.approx(sf, rel=8 / math.sqrt(n))
    rs = ratio_of_means(smoothen(a, 2 ** 3), smoothen(b, 2 ** 6), warn=False, rng=seed)
    assert 6 <= rs.k <= 8
    assert np.all(np.abs(q - rs.pquantile([0.16, 0.5, 0.84])) <= 2 * sf)
    assert abs(rs.f - f) <= 2 * sf and abs(rs.sigma_f - sf) <= 2 * sf
    pe, pe_err = rs                               # unpacks as (f, sigma_f)
    assert (pe, pe_err) == (rs.f, rs.sigma_f)


def test_ratio_of_means_documented_example():
    """The example in the reference's NamedTuple docstring (convenience.jl:144-152):
    ratio_of_means(1 .+ sin.(1:0.1:11), 2 .+ sin.(2:0.1:12)) has f = 0.560532,
    sigma_f = 0.0875548, k = 4 and 12 blocks, with blocking successful; the Monte Carlo median
    printed there, 0.581549 (+0.0812, -0.0926), is one draw of the sampled ratio."""
    from rimugpu.stats import ratio_of_means
    t = np.round(np.arange(101) * 0.1, 10)
    r = ratio_of_means(1 + np.sin(1 + t), 2 + np.sin(2 + t), warn=False, rng=0)
    assert round(r.f, 6) == 0.560532 and round(r.sigma_f, 7) == 0.0875548
    assert (r.k, r.blocks, r.success) == (4, 12, True)
    val, lo, hi = r.val_and_errs()
    assert val == pytest.approx(0.581549, abs=0.01)
    assert lo == pytest.approx(0.0926, abs=0.01) and hi == pytest.approx(0.0812, abs=0.01)


def test_ratio_of_means_edge_cases():
    """test/StatsTools.jl:65-109: blocks * 2^(k-1) <= n; a ratio of two zero-mean normal
    series (a Cauchy-like ratio) has a 95 % interval containing 0; zero-variance series give
    value and errors 0, and the ratio of two constant series is exact."""
    from rimugpu.stats import ratio_of_means
    rng = np.random.default_rng(17)
    br = ratio_of_means(rng.random(2000), rng.random(2000), alpha=0.05, warn=False, rng=1)
    assert br.blocks * 2 ** (br.k - 1) <= 2000
    r = ratio_of_means(rng.normal(size=2000), rng.normal(size=2000), warn=False, rng=2)
    q95 = r.pquantile([0.025, 0.975])
    assert q95[0] < 0 < q95[1]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        r0 = ratio_of_means([0, 0, 0, 0, 0, 0], [1, 1, 1, 1, 1, 2])
        assert r0.val_and_errs() == (0.0, 0.0, 0.0)
        assert tuple(r0) == (0.0, 0.0)
        r1 = ratio_of_means(np.ones(2000), np.ones(2000))
        assert tuple(r1) == (1.0, 0.0) and np.var(r1.ratio) == 0
        assert not r1.success
        rz = ratio_of_means(np.zeros(100), np.zeros(100))     # no projector weight at all
        assert math.isnan(rz.f)
