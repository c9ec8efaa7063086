"""pimc_blocking_se (host code of the library, no GPU): the blocking analysis
against a NumPy statement of the same algorithm, and its error bars
against series whose correlation is known.

The reference itself has no error analysis (it writes block averages,
mc_main.cc:764-795); the checks are the published properties of the method
(Flyvbjerg and Petersen 1989; Jonsson 2018): for an AR(1) series
x_k = phi x_{k-1} + e_k the statistical inefficiency is (1 + phi)/(1 - phi),
and a 95 % interval built from the error covers the true mean about 95 % of
the time.
"""
import numpy as np
import pytest
from scipy.stats import chi2

import pimc_gb300 as G


def blocking_np(x):
    x = np.asarray(x, dtype=np.float64)
    d = int(np.floor(np.log2(len(x))))
    b = x[len(x) - 2 ** d:].copy()
    mu = b.mean()
    s, g = np.zeros(d), np.zeros(d)
    for i in range(d):
        m = len(b)
        s[i] = np.sum((b - mu) ** 2) / m
        g[i] = np.sum((b[:-1] - mu) * (b[1:] - mu)) / m
        b = 0.5 * (b[0::2] + b[1::2])
    n_i = 2.0 ** (d - np.arange(d))
    M = np.cumsum((n_i * (g / s) ** 2)[::-1])[::-1]
    level = d - 1
    for j in range(d):
        if M[j] < chi2.ppf(0.99, d - j):
            level = j
            break
    return mu, np.sqrt(s[level] / 2.0 ** (d - level)), np.sqrt(s[0] / 2.0 ** d), 2 ** level


def ar1(rng, n, phi, mu=3.0):
    e = rng.normal(size=n)
    x = np.empty(n)
    x[0] = e[0] / np.sqrt(1 - phi * phi)
    for k in range(1, n):
        x[k] = phi * x[k - 1] + e[k]
    return x + mu


@pytest.mark.parametrize("phi,n", [(0.0, 5000), (0.5, 9000), (0.9, 1 << 15), (0.97, 70000)])
def test_matches_numpy_statement(phi, n):
    x = ar1(np.random.default_rng(int(phi * 100) + n), n, phi)
    r = G.blocking_se(x)
    mu, se, se0, blk = blocking_np(x)
    assert abs(r["mean"] - mu) <= 1e-12 * abs(mu)
    assert abs(r["se"] - se) <= 1e-12 * se and abs(r["se_naive"] - se0) <= 1e-12 * se0
    assert r["block"] == blk and r["n"] == 2 ** int(np.floor(np.log2(n)))


def test_inefficiency_of_ar1():
    rng = np.random.default_rng(5)
    for phi in (0.0, 0.8, 0.95):
        gs = [G.blocking_se(ar1(rng, 1 << 16, phi))["g"] for _ in range(6)]
        want = (1 + phi) / (1 - phi)
        assert 0.7 * want <= np.mean(gs) <= 1.3 * want, (phi, gs, want)


def test_coverage():
    rng = np.random.default_rng(9)
    hits = 0
    trials = 300
    for _ in range(trials):
        r = G.blocking_se(ar1(rng, 4096, 0.9, mu=0.0))
        hits += abs(r["mean"]) <= 1.96 * r["se"]
    assert 0.88 <= hits / trials <= 0.99, hits / trials


def test_rejects_short_and_nonfinite():
    with pytest.raises(G.PimcError):
        G.blocking_se(np.ones(15))
    x = np.ones(64)
    x[3] = np.nan
    with pytest.raises(G.PimcError):
        G.blocking_se(x)
