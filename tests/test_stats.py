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
