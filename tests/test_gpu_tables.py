"""The GPU propagator-table generators (pimc_linden, pimc_asymrho) against
the oracle's restatements of linear_prop/linden.f and nmv_prop/asymrho.f and
against the reference's own generator outputs (8 significant digits,
tests/golden/tables.npz)."""
import os

import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TAB = np.load(os.path.join(HERE, "golden", "tables.npz"))


def _maxchi(iphi):
    return np.where(iphi <= 90, iphi, np.where(iphi <= 180, 180 - iphi, np.where(iphi <= 270, iphi - 180, 360 - iphi)))


@pytest.mark.parametrize("iodevn", [-1, 0, 1])
def test_linden_matches_oracle(iodevn):
    """Many (T, slices) tables in one call; the same double operations in the
    same order as the oracle: equal to 1e-15 of each column's scale."""
    T = np.array([0.37, 0.5, 1.2, 2.0, 100.0])
    ns = np.array([128, 64, 256, 32, 4])
    B, npt = 0.39021, 1500
    got = G.linden(T, ns, B, npt, iodevn)
    for t in range(len(T)):
        ref = O.linden(T[t], int(ns[t]), B, npt, iodevn)
        for c in range(4):
            scale = np.max(np.abs(ref[c]))
            assert np.max(np.abs(got[t, c] - ref[c])) <= 1e-15 * scale, (t, c)


@pytest.mark.parametrize("key", ["co2", "n2o"])
def test_linden_matches_reference_tables(key):
    T, ns, B, npt = TAB["linden_%s_params" % key]
    got = G.linden([T], [int(ns)], B, int(npt))[0]
    rows = TAB["linden_%s_rows" % key]
    g = TAB["linden_%s_table" % key].T
    for c in range(4):
        err = np.abs(got[c, rows] - g[c])
        assert np.all(err <= 1e-8 * np.abs(g[c]) + 1e-9 * np.max(np.abs(g[c])))


def test_asymrho_matches_reference_slab():
    """The theta = 10 degree slab of nmv_prop/a-run (maxj 66): the propagator
    at every sampled point, the energy estimators where the propagator is
    above its cancellation noise, and the partition functions of the log."""
    p = TAB["asym_params"]
    rho, erot, esq, info = G.asymrho(p[0], int(p[1]), int(p[2]), int(p[3]), int(p[3]), p[4:7], int(p[7]))
    np.testing.assert_allclose(info, TAB["asym_info"], rtol=0, atol=6e-7)
    idx, vals, mx = TAB["asym_idx"], TAB["asym_vals"], TAB["asym_maxabs"]
    flat = [a[0].ravel()[idx] for a in (rho, erot, esq)]
    err = np.abs(flat[0] - vals[0])
    tol = 6e-8 * np.abs(vals[0]) + 1e-9 * mx[0]       # E15.8: 8 digits after "0."
    assert np.all(err <= tol), np.max(err / tol)
    big = np.abs(vals[0]) > 1e-4 * mx[0]
    for k in (1, 2):
        err = np.abs(flat[k][big] - vals[k][big])
        tol = 6e-8 * np.abs(vals[k][big]) + 1e-9 * mx[k]
        assert np.all(err <= tol), (k, np.max(err / tol))


@pytest.mark.parametrize("iodevn", [-1, 0, 1])
def test_asymrho_matches_oracle(iodevn):
    """A water-like top (A, B, C = 27.9, 14.5, 9.3 cm^-1) at 0.74 K with 2048
    slices, J <= 30: full slabs at four thetas against the oracle's state sums
    at points of the computed part of the grid; the symmetric copies of
    asymrho.f:636-709 equal their sources exactly."""
    abc = (27.9, 14.5, 9.3)
    ths = [0, 45, 90, 180]
    parts = [G.asymrho(0.74, 2048, iodevn, th, th, abc, 30) for th in ths]
    info = parts[0][3]
    rho, erot, esq = (np.zeros((181, 361, 361)) for _ in range(3))
    for th, (r_, e_, s_, _) in zip(ths, parts):
        rho[th], erot[th], esq[th] = r_[0], e_[0], s_[0]
    rng = np.random.default_rng(3)
    ith, iphi, ichi = [], [], []
    for th in ths:
        ph = rng.integers(0, 361, 6)
        ch = np.array([rng.integers(0, m + 1) for m in _maxchi(ph)])
        ith += [th] * 6; iphi += list(ph); ichi += list(ch)
    ith, iphi, ichi = map(np.array, (ith, iphi, ichi))
    r, e, s, oinfo = O.asymrho_points(0.74, 2048, iodevn, abc, 30, ith, iphi, ichi)
    # Cv = (<E^2> - <E>^2)/(kT)^2 cancels to noise of (E/kT)^2 where one state dominates
    kt = 0.6950356 * 0.74
    atol = np.zeros(15)
    for i in (2, 5, 8):
        atol[i] = 1e-15 * (max(abs(oinfo[i - 1]), 1.0) / kt) ** 2
    assert np.all(np.abs(info - oinfo) <= 1e-12 * np.abs(oinfo) + atol), (info, oinfo)
    scale = np.max(np.abs(rho[ths]))
    assert np.all(np.abs(rho[ith, iphi, ichi] - r) <= 1e-10 * scale)
    big = np.abs(r) > 1e-6 * scale
    for got, ref in ((erot, e), (esq, s)):
        g = got[ith, iphi, ichi][big]
        assert np.all(np.abs(g - ref[big]) <= 1e-8 * np.abs(ref[big]) + 1e-12 * np.max(np.abs(ref[big]))), \
            np.max(np.abs(g - ref[big]) / np.abs(ref[big]))
    # copies: (phi, chi) -> (chi, phi) of the last loop, for chi >= phi
    for th in ths:
        a = rho[th]
        iu = np.triu_indices(361)
        np.testing.assert_array_equal(a[iu], a.T[iu])
