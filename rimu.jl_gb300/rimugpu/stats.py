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


def x_by_y_linear(mu_x, mu_y, sigma_x, sigma_y, rho):
    """Ratio mu_x / mu_y of two correlated normal variables and its standard deviation by linear
    error propagation (x_by_y_linear, ratio_of_means.jl:166-171); rho is the covariance of x
    and y.  A variance that rounding makes slightly negative gives 0."""
    mu_x, mu_y = np.float64(mu_x), np.float64(mu_y)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        f = mu_x / mu_y
        var = (sigma_x / mu_y) ** 2 + (mu_x * sigma_y / mu_y ** 2) ** 2 - 2 * rho * mu_x / mu_y ** 3
    return float(f), float(np.sqrt(var)) if not var < 0 else 0.0


@dataclass
class RatioBlockingResult:
    """Result of ratio_of_means (RatioBlockingResult, ratio_of_means.jl:3-31): Monte Carlo
    samples of the ratio (`ratio`), the ratio of the means `f`, its linear-propagation error
    `sigma_f`, the denominator's coefficient of variation `delta_y` (the normal approximation
    holds for |delta_y| < 0.1), the blocking level k (k - 1 blocking steps), the number of
    blocks, and whether both blocking analyses succeeded.  Unpacks as (f, sigma_f)."""
    ratio: np.ndarray
    f: float
    sigma_f: float
    delta_y: float
    k: int
    blocks: int
    success: bool

    def __iter__(self):
        yield self.f
        yield self.sigma_f

    def pmedian(self) -> float:
        return float(np.median(self.ratio))

    def pquantile(self, q):
        return np.quantile(self.ratio, q)

    def val_and_errs(self, n=1):
        """Median and the distances to the quantiles that bound the central erf(n/sqrt 2)
        probability (val_and_errs, convenience.jl:99-107)."""
        p = math.erf(n / math.sqrt(2))
        q1, q2, q3 = self.pquantile([(1 - p) / 2, 0.5, 1 - (1 - p) / 2])
        return float(q2), float(q2 - q1), float(q3 - q2)


def ratio_estimators(x, y, k=None, corrected=True, mc_samples=2000, rng=None):
    """ratio_estimators (ratio_of_means.jl:196-230): after k - 1 blocking steps of both series,
    the means, the variances and the covariance of the means, Monte Carlo samples of the ratio
    of a bivariate normal with those moments (a variable without variance stays at its mean),
    the linear estimate and delta_y.  Returns (samples, f, sigma_f, delta_y, n)."""
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    for _ in range((k or 1) - 1):
        x, y = blocker(x), blocker(y)
    n = len(x)
    mu_x, mu_y = float(np.mean(x)), float(np.mean(y))
    dd = int(corrected)
    var_x = float(np.sum((x - mu_x) ** 2) / (n - dd)) / n
    var_y = float(np.sum((y - mu_y) ** 2) / (n - dd)) / n
    rho = float(np.sum((x - mu_x) * (y - mu_y)) / (n - dd)) / n
    f, sigma_f = x_by_y_linear(mu_x, mu_y, math.sqrt(var_x), math.sqrt(var_y), rho)
    rng = np.random.default_rng(rng)
    z = rng.standard_normal((2, int(mc_samples)))
    eps = math.sqrt(np.finfo(float).eps)
    if abs(var_x) < eps or abs(var_y) < eps:     # singular: independent (or constant) draws
        px = mu_x + math.sqrt(var_x) * z[0]
        py = mu_y + math.sqrt(var_y) * z[1]
    else:
        c = np.linalg.cholesky(np.array([[var_x, rho], [rho, var_y]]))
        px = mu_x + c[0, 0] * z[0]
        py = mu_y + c[1, 0] * z[0] + c[1, 1] * z[1]
    with np.errstate(divide="ignore", invalid="ignore"):
        samples = px / py
        delta_y = math.sqrt(var_y) / mu_y if mu_y != 0 else math.inf
    return samples, f, sigma_f, delta_y, n


def ratio_of_means(num, denom, alpha=0.01, corrected=True, mc_samples=2000, skip=0, warn=True,
                   rng=None) -> RatioBlockingResult:
    """ratio_of_means (ratio_of_means.jl:126-157): both series are blocked to the larger of
    the levels their M-tests pick, the error of the ratio is propagated linearly and by Monte
    Carlo sampling, and `f` is the ratio of the unblocked means.  A zero denominator mean gives
    a NaN or infinite ratio, as the floating-point division does."""
    num = np.asarray(num, float)[skip:]
    den = np.asarray(denom, float)[skip:]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        bn = blocking_analysis(num, alpha=alpha, corrected=corrected)
        bd = blocking_analysis(den, alpha=alpha, corrected=corrected)
    success = bn.k >= 0 and bd.k >= 0
    if warn and not success:
        warnings.warn(f"Blocking failed in `ratio_of_means`: k = {(bn.k, bd.k)}")
    k = max(bn.k, bd.k)
    samples, _, sigma_f, delta_y, n = ratio_estimators(num, den, k if k > 1 else None, corrected,
                                                      mc_samples, rng)
    if warn and abs(delta_y) >= 0.1:
        warnings.warn("Large coefficient of variation in `ratio_of_means`: |delta_y| >= 0.1")
    with np.errstate(divide="ignore", invalid="ignore"):
        f = float(np.float64(bn.mean) / np.float64(bd.mean))
    return RatioBlockingResult(samples, f, sigma_f, delta_y, k, n, success)


def projected_energy(df, hproj="hproj", vproj="vproj", skip=0, **kw):
    """projected_energy (reweighting.jl:721-726): ratio of means of hproj and vproj."""
    return ratio_of_means(df[hproj], df[vproj], skip=skip, **kw)
