"""The oracle's restatements of the propagator-table generators
(oracle/orc_tables.c) against the reference's own generator outputs:
linear_prop/linden.f tables shipped with the examples, the theta = 10 degree
slab of nmv_prop/asymrho.f with its log (tests/golden/make_tables_golden.py).
Those files carry 8 significant digits."""
import os

import numpy as np
import pytest

import oracle as O
import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
TAB = np.load(os.path.join(HERE, "golden", "tables.npz"))


def _digits8(got, ref, maxabs, rel=1e-8, frac=1e-9):
    err = np.abs(np.asarray(got) - np.asarray(ref))
    assert np.all(err <= rel * np.abs(ref) + frac * maxabs), np.max(err / (rel * np.abs(ref) + frac * maxabs))


@pytest.mark.parametrize("key", ["co2", "n2o"])
def test_linden_matches_reference_tables(key):
    T, ns, B, npt = TAB["linden_%s_params" % key]
    t = O.linden(T, int(ns), B, int(npt))
    rows = TAB["linden_%s_rows" % key]
    g = TAB["linden_%s_table" % key].T
    for c in range(4):
        _digits8(t[c, rows], g[c], np.max(np.abs(g[c])))
    # the same sums as the numpy restatement used to build the workloads
    tau = 1.4387752224 / (T * ns)
    r, e, s = W.linden_exarho(t[0], tau, B, int(ns))
    np.testing.assert_array_equal(t[1], r)
    np.testing.assert_array_equal(t[2], e)
    np.testing.assert_array_equal(t[3], s)


def test_asymrho_eigenvalues_and_partition_functions():
    p = TAB["asym_params"]
    abc = p[4:7]
    eng = np.sort(O.asymrho_energies(2, abc))
    np.testing.assert_allclose(eng, TAB["asym_log_eigs"], atol=6e-5)      # printed f9.4
    r, e, s, info = O.asymrho_points(p[0], int(p[1]), int(p[2]), abc, int(p[7]), [10], [0], [0])
    np.testing.assert_allclose(info, TAB["asym_info"], rtol=0, atol=6e-7)          # printed f12.6


def test_asymrho_points_match_reference_slab():
    """A few points of the theta = 10 slab where the propagator is not at its
    cancellation noise (|rho| > 1e-3 max), all three columns."""
    p = TAB["asym_params"]
    idx, vals, mx = TAB["asym_idx"], TAB["asym_vals"], TAB["asym_maxabs"]
    iphi, ichi = idx // 361, idx % 361
    # points of the computed (fundamental) part of the grid (asymrho.f:530-541)
    maxchi = np.where(iphi <= 90, iphi, np.where(iphi <= 180, 180 - iphi, np.where(iphi <= 270, iphi - 180, 360 - iphi)))
    cand = np.flatnonzero((np.abs(vals[0]) > 1e-3 * mx[0]) & (ichi <= maxchi))
    pick = cand[np.linspace(0, len(cand) - 1, 5).astype(int)]
    r, e, s, info = O.asymrho_points(p[0], int(p[1]), int(p[2]), p[4:7], int(p[7]), np.full(len(pick), int(p[3])),
                                     iphi[pick], ichi[pick])
    for k, got in enumerate((r, e, s)):
        _digits8(got, vals[k][pick], mx[k], rel=6e-8, frac=1e-9)   # E15.8: 8 digits after "0."
