"""Blocking analysis of time series (src/StatsTools/blocking.jl, variances.jl).

Flyvbjerg-Petersen reblocking with Jonsson's M-test for choosing the blocking level, used
to attach error bars to the shift and projected-energy estimators.
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass

import numpy as np


@dataclass
class BlockingResult:
    mean: float
    err: float
    err_err: float
    p_cov: float
    k: int
    blocks: int


def blocker(v: np.ndarray) -> np.ndarray:
    """Mean of adjacent pairs; an odd last point is dropped (blocking.jl:254-261)."""
    n = len(v) // 2
    return (v[0:2 * n:2] + v[1:2 * n:2]) / 2


def autocovariance(v, h, corrected=True, mean=None):
    """variances.jl:8-16."""
    mean = np.mean(v) if mean is None else mean
    n = len(v)
    return float(np.sum((v[: n - h] - mean) * (v[h:] - mean)) / (n - int(corrected)))


def blocks_with_m(v, corrected=True):
    """blocks_with_m (blocking.jl:294-325)."""
    v = np.asarray(v, dtype=float)
    n_steps = int(math.floor(math.log2(len(v))))
    out = {k: [] for k in ("blocks", "mean", "std_err", "std_err_err", "p_cov", "mj")}
    for _ in range(n_steps):
        n = len(v)
        m = float(np.mean(v))
        var = float(np.sum((v - m) ** 2) / (n - int(corrected)))
        gamma = autocovariance(v, 1, corrected, m)
        # Eq. (12) of Jonsson; a series without variance gives 0/0 = NaN as in the reference,
        # so the M-test fails on it instead of passing
        mj = n * ((n - 1) * var / (n ** 2) + gamma) ** 2 / (var ** 2) if var > 0 else math.nan
        se = math.sqrt(var / n)
        out["blocks"].append(n)
        out["mean"].append(m)
        out["std_err"].append(se)
        out["std_err_err"].append(se / math.sqrt(2 * (n - 1)))
        out["p_cov"].append(float(np.sum((v - m) ** 2) / (n - int(corrected))) / n)
        out["mj"].append(mj)
        v = blocker(v)
    return out


def mtest(mj, alpha=0.01) -> int:
    """Jonsson's M-test (blocking.jl:274-286); returns the 1-based level or -1."""
    from scipy.stats import chi2
    m = np.cumsum(np.asarray(mj)[::-1])[::-1]
    k = 1
    while k <= len(m) - 1:
        if m[k - 1] < chi2.isf(alpha, k):
            return k
        k += 1
    return -1


def blocking_analysis(v, alpha=0.01, corrected=True, skip=0) -> BlockingResult:
    """blocking_analysis (blocking.jl:134-159)."""
    v = np.asarray(v, dtype=float)[skip:]
    if len(v) < 2:
        warnings.warn("Attempted blocking on an empty vector." if len(v) == 0 else
                      f"Attempted blocking on a vector of length {len(v)}.")
        return BlockingResult(float(v[0]) if len(v) else 0.0, math.nan, math.nan, math.nan, -1, len(v))
    nt = blocks_with_m(v, corrected)
    k = mtest(nt["mj"], alpha)
    if k < 0:
        warnings.warn("Hypothesis testing failed during blocking_analysis. "
                      "Try using more time steps!")
        return BlockingResult(nt["mean"][0], math.nan, math.nan, math.nan, k, 0)
    return BlockingResult(nt["mean"][0], nt["std_err"][k - 1], nt["std_err_err"][k - 1],
                          nt["p_cov"][k - 1], k, nt["blocks"][k - 1])


def mean_and_se(v, **kw):
    r = blocking_analysis(v, **kw)
    return r.mean, r.err


def shift_estimator(df, shift="shift", skip=0):
    """shift_estimator (reweighting.jl:739-743) without reweighting."""
    return blocking_analysis(np.asarray(df[shift]), skip=skip)


def ratio_of_means(num, denom, skip=0):
    """Ratio of means with a first-order (delta method) error from blocked series;
    a simplified ratio_of_means (ratio_of_means.jl:126)."""
    num = np.asarray(num, float)[skip:]
    den = np.asarray(denom, float)[skip:]
    rn, rd = blocking_analysis(num), blocking_analysis(den)
    if rd.mean == 0:             # the projector never saw a walker: no estimate
        return math.nan, math.nan
    r = rn.mean / rd.mean
    k = max(rn.k, rd.k, 1)
    b = 2 ** (k - 1)
    nb = len(num) // b
    if nb >= 2:
        bn = num[: nb * b].reshape(nb, b).mean(1)
        bd = den[: nb * b].reshape(nb, b).mean(1)
        cov = np.cov(bn, bd)
        var = (cov[0, 0] / rd.mean ** 2 - 2 * r * cov[0, 1] / rd.mean ** 2
               + r ** 2 * cov[1, 1] / rd.mean ** 2) / nb
        err = math.sqrt(max(var, 0.0))
    else:
        err = math.nan
    return r, err


def projected_energy(df, hproj="hproj", vproj="vproj", skip=0):
    """projected_energy (reweighting.jl:721-726): ratio of means of hproj and vproj."""
    return ratio_of_means(df[hproj], df[vproj], skip)
