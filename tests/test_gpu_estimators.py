"""GPU estimators beyond the energies: the pair-density histograms of
GetPotEnergy_Densities (mc_estim.cc:500-687, bins :1233-1286), the exchange
cycle lengths of GetExchangeLength (:1997-2019) and the superfluid area
estimators GetAreaEstimators / GetAreaEstim3D (:2087-2594), through the C ABI.

Histogram counts and cycle lengths are integers and must match exactly.  The
area sums are FP64 sums of N_bosons * P signed terms summed in another order
than the reference's; their bound is 1e-10 of the terms' magnitude."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W
from _common import area_scales, check_area, dense_hist, golden, golden_cases

pytestmark = pytest.mark.gpu
RTOL = 1e-10


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name", golden_cases())
def test_estimators_match_reference_fixture(name, mixed):
    w, d, _ = golden(name)
    if "perm" not in d:
        pytest.skip("no bosons in this system")
    s = G.Sampler(w, mixed=mixed)
    s.set_state(d["coords1"], d["angles1"], d["perm"])
    s.set_option(G.OPT_DENSITIES, 1)
    est = s.estimators()
    assert est[1] == pytest.approx(float(d["dens_pot"]), rel=RTOL, abs=1e-12)
    g1, g2, g3 = s.densities_read()
    np.testing.assert_array_equal(g1, dense_hist(d, "g1", g1.shape))
    np.testing.assert_array_equal(g2, dense_hist(d, "g2", g2.shape))
    np.testing.assert_array_equal(g3, dense_hist(d, "g3", g3.shape))
    # a second sample of the same configuration doubles every count; reset clears
    s.densities_accumulate()
    h1, h2, h3 = s.densities_read()
    np.testing.assert_array_equal(h1, 2 * g1)
    np.testing.assert_array_equal(h3, 2 * g3)
    s.densities_reset()
    z1, z2, z3 = s.densities_read()
    assert z1.sum() == 0 and z2.sum() == 0 and z3.sum() == 0
    # exchange cycles add into the caller's array like _ploops
    pl = s.exchange_lengths()
    np.testing.assert_array_equal(pl, d["ploops"])
    s.exchange_lengths(pl)
    np.testing.assert_array_equal(pl, 2 * d["ploops"])
    s_area, s_inert = area_scales(w, d["coords1"], d["masses"])
    if "area2d" in d:
        check_area(s.area_estimators(), d["area2d"], s_area, s_inert, False)
    else:
        with pytest.raises(G.PimcError):
            s.area_estimators()             # needs a linear dopant
    for fr in (0, 1):
        check_area(s.area_estim3d(fr, d["masses"]), d["area3d"][fr], s_area, s_inert, True)
    s.close()


@pytest.mark.parametrize("which", ["config0", "config1"])
def test_estimators_after_production_passes(which):
    """At the benchmark sizes (8 He around the linear rotor at P=512; 64 pH2
    around the top at P=1024): sample with the production schedule, then
    compare the GPU's estimators of the sampled path, under a random boson
    permutation, with the oracle's on the same path."""
    if which == "config0":
        w = W.config0()
        masses = np.array([W.MASSES["He4"], W.MASSES["CO2"]])
    else:
        w = W.config1(grid3d=(60, 181, 91), griddens=(19, 37, 37))
        masses = np.array([W.MASSES["H2"], W.MASSES["SO2"]])
    s = G.Sampler(w)
    s.set_option(G.OPT_DENSITIES, 1)
    s.run_passes(2, seed=99)
    c, a, co, p = s.get_state()
    nbos = w.types[0]["numb"]
    perm = np.arange(w.natoms, dtype=np.int32)
    perm[:nbos] = np.random.default_rng(7).permutation(nbos)
    s.set_state(c, a, perm)
    s.densities_reset()
    s.densities_accumulate()
    g1, g2, g3 = s.densities_read()
    o = O.Oracle(w)
    o.set_state(c, a, perm)
    _, r1, r2, r3 = o.densities()
    np.testing.assert_array_equal(g1, r1)
    np.testing.assert_array_equal(g2, r2)
    np.testing.assert_array_equal(g3, r3)
    assert g1.sum() + g2.sum() + g3.sum() > 0
    np.testing.assert_array_equal(s.exchange_lengths(), o.exchange_lengths(nbos))
    s_area, s_inert = area_scales(w, c, masses)
    if w.types[1]["molecule"] == 1:
        got, ref = s.area_estimators(), o.area_estimators()
        check_area(got, ref, s_area, s_inert, False)
    for fr in (0, 1):
        got, ref = s.area_estim3d(fr, masses), o.area_estim3d(fr, masses)
        check_area(got, ref[3:], s_area, s_inert, True)
    s.close()


def test_relative_euler_histograms_match_oracle_angles():
    """GetRotE3D's binning of the relative Euler angles of adjacent
    rotational slices (mc_estim.cc:1023-1057) on a sampled asymmetric-top
    path: the device histograms equal the binning of the oracle's rotden
    relative angles of the same slices."""
    w = W.config1(seed=12, nslices=32, nrotslices=8, n_h2=6, grid3d=(30, 37, 19), griddens=(19, 37, 37))
    s = G.Sampler(w)
    s.set_option(G.OPT_DENSITIES, 1)
    s.run_passes(3, seed=5)
    c, a, co, p = s.get_state()
    s.densities_reset()
    s.densities_accumulate()
    t, ph, ch = s.rel_euler_read()
    s.close()
    o = O.Oracle(w)
    o.set_state(c, a, p)
    first = sum(tp["numb"] for tp in w.types if tp["molecule"] == 0)
    off, Q = first * w.nslices, w.nrotslices
    dth, dch = np.pi / (G.BINST - 1), 2.0 * np.pi / (G.BINSC - 1)
    rt, rp, rc = np.zeros(G.BINST), np.zeros(G.BINSC), np.zeros(G.BINSC)
    for it0 in range(Q):
        e = [(a[0, off + i], np.arccos(a[1, off + i]), a[2, off + i]) for i in (it0, (it0 + 1) % Q)]
        _, rel, _, _, _ = o.rotden(e[0], e[1])
        for hist, v, d in ((rt, rel[1], dth), (rp, rel[0], dch), (rc, rel[2], dch)):
            b = int(np.floor(v / d))
            if 0 <= b < len(hist):
                hist[b] += 1
    np.testing.assert_array_equal(t, rt)
    np.testing.assert_array_equal(ph, rp)
    np.testing.assert_array_equal(ch, rc)
    assert t.sum() == Q
