"""The matched-SE measurement's host arithmetic in bench.py (no GPU): the
pooled statistical inefficiency, the time-to-target-SE formula and the ratio
estimator that scales the plain path's sampled pass times to all replicas.

Checks against series and samples whose answers are known: an AR(1) series
x_k = phi x_{k-1} + e_k has g = (1 + phi) / (1 - phi); pass times exactly
proportional to the work units scale without error; with noise, the
estimator's interval covers the true total at about its nominal rate."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import bench  # noqa: E402


def ar1_matrix(rng, npass, nrep, phi):
    x = np.empty((npass, nrep))
    x[0] = rng.normal(size=nrep) / np.sqrt(1 - phi * phi)
    for k in range(1, npass):
        x[k] = phi * x[k - 1] + rng.normal(size=nrep)
    return x


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.8])
def test_pooled_inefficiency_of_ar1(phi):
    """Long series: within 15 % of (1 + phi) / (1 - phi)."""
    rng = np.random.default_rng(int(phi * 10) + 1)
    g = bench.pooled_inefficiency(ar1_matrix(rng, 1024, 128, phi))
    want = (1 + phi) / (1 - phi)
    assert abs(g - want) <= 0.15 * want, (g, want)


def test_pooled_inefficiency_is_low_on_short_series():
    """Each replica's series is centred on its own mean, which biases g low
    when the series is not much longer than g (at 64 passes and phi = 0.8
    about half the true 9).  The matched-SE ratios do not depend on it where
    the arms share one g (config 4) or make the same moves (the dimers'
    unscreened arms); the reported pass counts are then lower bounds."""
    rng = np.random.default_rng(7)
    g_short = bench.pooled_inefficiency(ar1_matrix(rng, 64, 512, 0.8))
    g_long = bench.pooled_inefficiency(ar1_matrix(rng, 1024, 128, 0.8))
    assert g_short < g_long < 9.0 * 1.15


def test_matched_time_to_se():
    arms = {"a": {"g": 2.0, "var": np.ones(4), "pass_ms": 10.0},
            "b": {"g": 4.0, "var": np.ones(4) * 1.1, "pass_ms": 1.0}}
    out = bench.matched(1000.0, 3.0, arms, c=0.05)
    assert out["plain"]["passes"] == pytest.approx(3.0 / 0.0025)
    assert out["plain"]["seconds"] == pytest.approx(3.0 / 0.0025 * 1.0)
    assert out["a"]["passes"] == pytest.approx(2.0 / 0.0025)
    assert out["a"]["seconds"] == pytest.approx(2.0 / 0.0025 * 0.01)
    # the ratio is (g_plain t_plain) / (g_arm t_arm); the variances only reported
    assert out["a"]["vs_plain"] == pytest.approx(round(3.0 * 1000.0 / (2.0 * 10.0), 2))
    assert out["b"]["vs_plain"] == pytest.approx(round(3.0 * 1000.0 / (4.0 * 1.0), 2))
    assert out["a"]["var_ratio"] == pytest.approx(round(1.0 / 1.05, 4))


class _W:
    def __init__(self, bm, natoms):
        self._bm = bm
        self.natoms = natoms

    def bead_moves_per_pass(self):
        return self._bm


def _family(rng, n=512):
    return [_W(float(rng.integers(1000, 100000)), int(rng.integers(1, 40))) for _ in range(n)]


def test_ratio_estimator_exact_when_proportional():
    rng = np.random.default_rng(3)
    ws = _family(rng)
    idx = rng.choice(len(ws), size=24, replace=False)
    rate = 2.5e-6                                   # ms per work unit
    ts = [rate * bench.work_units(ws[i]) for i in idx]
    total, se = bench.scaled_total(ws, idx, ts)
    true = rate * sum(bench.work_units(w) for w in ws)
    assert total == pytest.approx(true, rel=1e-12)
    assert se == pytest.approx(0.0, abs=1e-9 * true)


def test_ratio_estimator_coverage():
    rng = np.random.default_rng(4)
    ws = _family(rng)
    units = np.array([bench.work_units(w) for w in ws], dtype=np.float64)
    times = 2.5e-6 * units * rng.lognormal(0.0, 0.3, size=len(ws))
    true = float(times.sum())
    hits, trials = 0, 400
    for _ in range(trials):
        idx = rng.choice(len(ws), size=24, replace=False)
        total, se = bench.scaled_total(ws, idx, times[idx])
        hits += abs(total - true) <= 1.96 * se
    assert 0.85 <= hits / trials <= 0.99, hits / trials
