"""Known-answer tests for the oracle's restatements of the Fortran leaves
(rotden.f, rotpro_sub.f, vcord.f, vcalc.f, caleng_tip4p_gg.f, vspher.f),
which cannot be compiled here, and live comparisons of the oracle's
table lookups with the reference's own C++ (skipped if oracle/_ref is absent)."""
import math

import numpy as np
import pytest

import oracle as O
import workloads as W


@pytest.fixture(scope="module")
def c1():
    w = W.config1(seed=3, nslices=16, nrotslices=4, n_h2=3, grid3d=(30, 181, 91), griddens=(19, 37, 37))
    return w, O.Oracle(w)


def _mat(e):
    m = np.zeros(9)
    O.lib().orc_matpre(O.dptr(np.ascontiguousarray(e, dtype=np.float64)), O.dptr(m))
    return m.reshape(3, 3)


def test_matpre_is_zyz_rotation():
    rng = np.random.default_rng(0)
    for _ in range(20):
        phi, th, chi = rng.uniform(0, 2 * np.pi), rng.uniform(0, np.pi), rng.uniform(0, 2 * np.pi)
        rz = lambda a: np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
        ry = lambda a: np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
        np.testing.assert_allclose(_mat([phi, th, chi]), rz(phi) @ ry(th) @ rz(chi), atol=1e-14)


def test_deleul_recovers_relative_rotation():
    rng = np.random.default_rng(1)
    for _ in range(50):
        e1 = [rng.uniform(0, 2 * np.pi), rng.uniform(0.1, 3.0), rng.uniform(0, 2 * np.pi)]
        e2 = [rng.uniform(0, 2 * np.pi), rng.uniform(0.1, 3.0), rng.uniform(0, 2 * np.pi)]
        rel = np.zeros(3)
        O.lib().orc_deleul(O.dptr(np.array(e1)), O.dptr(np.array(e2)), O.dptr(rel))
        np.testing.assert_allclose(_mat(rel), _mat(e1).T @ _mat(e2), atol=1e-9)
        assert 0 <= rel[0] <= 2 * np.pi and 0 <= rel[1] <= np.pi and 0 <= rel[2] <= 2 * np.pi


def test_rotden_first_order_interpolation(c1):
    """rotpro: value at the lower node plus one-sided first differences along
    chi, phi, theta times the fractional offsets (rotpro_sub.f:26-61); erot
    and esq divided by wno2k, wno2k^2 (rotden.f:28-29)."""
    w, o = c1
    tb = w.tables
    nth, nph, nch = tb["nth"], tb["nph"], tb["nch"]
    rho3 = tb["rhoprp"].reshape(nth, nph, nch)
    er3 = tb["erotpr"].reshape(nth, nph, nch)
    dth, dph, dch = 180.0 / (nth - 1), 360.0 / (nph - 1), 360.0 / (nch - 1)
    for ith, iph, ich, f in [(3, 5, 7, 0.3), (10, 20, 30, 0.6), (1, 1, 1, 0.25)]:
        th, ph, ch = (ith + f) * dth, (iph + f) * dph, (ich + f) * dch
        st, rel, rho, er, es = o.rotden([0.0, 0.0, 0.0], np.radians([ph, th, ch]))
        assert st == 0
        for arr, got, scale in ((rho3, rho, 1.0), (er3, er, 0.6950356)):
            v0 = arr[ith, iph, ich]
            expect = v0 + (arr[ith, iph, ich + 1] - v0) * f + (arr[ith, iph + 1, ich] - v0) * f \
                + (arr[ith + 1, iph, ich] - v0) * f
            assert got == pytest.approx(expect / scale, rel=1e-9)


def test_vcord_radial_linear_and_angles(c1):
    """vcalc's first-order interpolation: exact at nodes; linear in r between
    nodes; r in bohr (vcord.f:87); theta measured from the body z axis."""
    w, o = c1
    tb = w.tables
    vt = tb["vtable"]
    rstep = (tb["rvmax"] - tb["rvmin"]) / (tb["rgrd"] - 1)
    bohr = 0.529177249
    # atom on the body z axis (theta = 0) at node ir -> vtable[ir, 0, chi node]
    for ir in (2, 5, 11):
        rb = tb["rvmin"] + ir * rstep
        v, rad, the, chi = o.vcord([0.0, 0.0, 0.0], [0, 0, 0], [0, 0, rb * bohr])
        assert the == pytest.approx(0.0, abs=1e-7)
        assert v == pytest.approx(vt[ir, 0, 90 // 1 if tb["chgrd"] == 91 else 0], rel=1e-6)
        # half-way in r: mean of the two radial nodes (same angular node)
        v2, *_ = o.vcord([0.0, 0.0, 0.0], [0, 0, 0], [0, 0, (rb + 0.5 * rstep) * bohr])
        assert v2 == pytest.approx(0.5 * (vt[ir, 0, 90] + vt[ir + 1, 0, 90]), rel=1e-6)


def test_caleng_symmetry_and_formula():
    """caleng: swapping the two waters leaves the energy unchanged; the value
    matches an independent evaluation of the TIP4P-like terms with the LJ
    term scaled by 503 (kcal2k is an INTEGER parameter, caleng_tip4p_gg.f:36)."""
    rng = np.random.default_rng(7)
    sites = np.array([[0, 0, 0.06562], [0.7557, 0, -0.5223], [-0.7557, 0, -0.5223], [0, 0, -0.08438]])
    for _ in range(20):
        c1 = rng.normal(0, 0.2, 3); c2 = c1 + np.array([2.9, 0.3, -0.2]) + rng.normal(0, 0.1, 3)
        e1 = [rng.uniform(0, 6.28), rng.uniform(0.1, 3.0), rng.uniform(0, 6.28)]
        e2 = [rng.uniform(0, 6.28), rng.uniform(0.1, 3.0), rng.uniform(0, 6.28)]
        f = O.lib().orc_caleng
        E12 = f(O.dptr(c1), O.dptr(c2), O.dptr(np.array(e1)), O.dptr(np.array(e2)))
        E21 = f(O.dptr(c2), O.dptr(c1), O.dptr(np.array(e2)), O.dptr(np.array(e1)))
        assert E12 == pytest.approx(E21, rel=1e-12)
        s1 = c1 + sites @ _mat(e1).T
        s2 = c2 + sites @ _mat(e2).T
        O1, H11, H21, M1 = s1
        O2, H12, H22, M2 = s2
        d = lambda a, b: np.linalg.norm(a - b)
        roo = d(O1, O2)
        lj = 6.0e5 / roo**12 - 610.0 / roo**6
        qm, qh = -1.04, 0.52
        coul = (qm * qh * (1 / d(M1, H12) + 1 / d(M1, H22) + 1 / d(M2, H11) + 1 / d(M2, H21))
                + qm * qm / d(M1, M2)
                + qh * qh * (1 / d(H11, H12) + 1 / d(H11, H22) + 1 / d(H21, H12) + 1 / d(H21, H22)))
        assert E12 == pytest.approx(lj * 503.0 + coul * 3.1577465e5 * 0.52917721092, rel=1e-10)


def test_rsline_formula():
    rho, er = O.C.c_double(), O.C.c_double()
    O.lib().orc_rsline(0.39, 0.3, 0.02, O.C.byref(rho), O.C.byref(er))
    tau = 0.02 / 0.6950356
    r = (1 - 0.3) / (2 * 0.39 * tau)
    assert rho.value == pytest.approx(-r, rel=1e-14)
    assert er.value == pytest.approx((1 - r) / tau / 0.6950356, rel=1e-14)


def test_vspher_single_precision_conversion():
    w = W.config1(seed=3, nslices=16, nrotslices=4, n_h2=2, grid3d=(10, 19, 10), griddens=(7, 13, 13))
    tab = np.linspace(1.0, 2.0, 501)
    w.tables.update(sph_table=tab, sph_r0=3.0, sph_rmax=26.0, sph_rstep=0.046)
    o = O.Oracle(w)
    r = 5.0
    rb = r / float(np.float32(0.5291772))
    ir = int((rb - 3.0) / 0.046)
    expect = tab[ir] + (tab[ir + 1] - tab[ir]) / 0.046 * (rb - (3.0 + ir * 0.046))
    assert o.vspher(r) == pytest.approx(expect, rel=1e-14)
    assert o.vspher(0.1) == pytest.approx(tab[0])            # clamped below r0
    assert o.vspher(100.0) == pytest.approx(tab[500])        # clamped at rmax, no gradient


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here (oracle/ref_build.sh)")
def test_table_lookups_against_reference():
    """SPot1D incl. both extrapolations, LPot2D incl. linear extrapolation,
    SRotDens/Deriv/Esqrt incl. out-of-grid branches (mc_poten.cc:548-729)."""
    w = W.config0(seed=2, nslices=16, nrotslices=4, n_he=2, r2d_step=0.05, c2d_step=0.04)
    o = O.Oracle(w)
    r = O.Reference(w)
    rng = np.random.default_rng(5)
    for x in np.concatenate([rng.uniform(0.5, 35.0, 300), [1.0, 30.0, 0.9, 31.0]]):
        assert o.spot1d(x) == r.L.ref_spot1d(x, 0)
    for x, c in zip(rng.uniform(1.5, 21.0, 300), rng.uniform(-1.05, 1.05, 300)):
        assert o.lpot2d(x, c) == r.L.ref_lpot2d(x, c, 1)
    for g in np.concatenate([rng.uniform(-1.0, 1.0, 300), [-1.0, 1.0, 1.0000001, -1.0000001]]):
        for which in range(3):
            assert o.srotdens(g, which) == r.L.ref_srotdens(g, 1, which)
