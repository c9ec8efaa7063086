"""The oracle against the golden fixtures generated from the reference's own
C++ (tests/golden/make_golden.py).  CPU only; runs wherever the oracle builds."""
import numpy as np
import pytest

import oracle as O
from _common import (area_scales, check_area, dense_hist, golden, golden_cases, nrotors, replay_sequence,
                     rot_est_from_reference, rs_energy, rs_rotor_means)

RTOL = 1e-10   # FP64 parity bound of the hot path


@pytest.fixture(scope="module", params=golden_cases())
def case(request):
    w, d, M = golden(request.param)
    return request.param, w, d


def test_tables_regenerate(case):
    name, w, d = case
    for k, v in w.tables.items():
        if isinstance(v, np.ndarray):
            ref = d["tab_" + k]
            got = np.array([float(np.sum(v)), float(np.sum(np.abs(v))), float(v.ravel()[len(v.ravel()) // 3])])
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12, err_msg=k)


def test_energies(case):
    name, w, d = case
    o = O.Oracle(w)
    c0 = np.ascontiguousarray(d["coords0"])
    pos = d["pos"]
    for a in range(w.natoms):
        for j, it in enumerate(d["slices"]):
            assert o.pot_energy_slice(a, c0, it) == pytest.approx(d["e_slice"][a, j, 0], rel=RTOL, abs=1e-12)
            assert o.pot_energy_slice(a, pos, it) == pytest.approx(d["e_slice"][a, j, 1], rel=RTOL, abs=1e-12)
        assert o.pot_energy_path(a, c0) == pytest.approx(d["e_path"][a, 0], rel=RTOL, abs=1e-12)
        assert o.pot_energy_path(a, pos) == pytest.approx(d["e_path"][a, 1], rel=RTOL, abs=1e-12)


def test_rotor_energies(case):
    name, w, d = case
    if not w.rotation:
        pytest.skip("no rotational slices in this system")
    o = O.Oracle(w)
    rtype = [i for i, t in enumerate(w.types) if t["molecule"] != 0][0]
    roff = sum(t["numb"] for t in w.types[:rtype])
    nb = w.natoms * w.nslices
    for k in range(d["eul"].shape[0]):
        e = d["eul"][k]
        for j, it in enumerate(d["slices"]):
            if w.types[rtype]["molecule"] == 1:
                cos = np.zeros((3, nb))
                cos[0] = np.sin(e[1]) * np.cos(e[0]); cos[1] = np.sin(e[1]) * np.sin(e[0]); cos[2] = np.cos(e[1])
                got = o.pot_rot_energy(roff, cos, it)
            else:
                got = o.pot_rot_e3d(roff, e, it)
            assert got == pytest.approx(d["e_rot"][k, j], rel=RTOL, abs=1e-12)


def test_move_sequence(case):
    name, w, d = case
    o = O.Oracle(w)

    def bis(typ, t, g, u3):
        st, ds, lv, pos = o.bisection_move(typ, t, g, u3)
        assert st == 0
        return pos

    def mol(typ, u1, u2):
        st, dv, acc, pos = o.molecular_move(typ, u1, u2)
        assert st == 0
        return pos

    def rot(typ, ur):
        st, rd, acc, pos = o.rotations(typ, ur)
        assert st == 0
        return pos

    consumed = replay_sequence(d, bis, mol, rot)
    # random numbers consumed per call, generator by generator
    for (kind, typ, t), got, ref in zip(d["seq"], consumed, d["consumed"]):
        if kind == 0:
            assert got == (ref[3], ref[2])
        elif kind == 1:
            assert got == (ref[0], ref[1])
        else:
            assert got == ref[4]
    c, a, co, _ = o.get_state()
    np.testing.assert_allclose(c, d["coords1"], rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(a, d["angles1"], rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(co, d["cosine1"], rtol=RTOL, atol=1e-12)
    tot, acc = o.counters()
    np.testing.assert_array_equal(tot[:len(d["total"])], d["total"])
    np.testing.assert_array_equal(acc[:len(d["accep"])], d["accep"])
    # estimators of the final path (GetKinEnergy, GetPotEnergy_Densities, GetRot*)
    nonlinear = any(t["molecule"] == 2 for t in w.types)
    rot, esq, ets = o.rot_energy(nonlinear) if w.rotation else (0.0, 0.0, 0.0)
    got = np.array([o.kin_energy(), o.pot_energy_est(), rot, esq, ets])
    erot_ok, sq_ok = rot_est_from_reference(w)
    keep = [0, 1] + ([2] if erot_ok else []) + ([3, 4] if sq_ok else [])
    np.testing.assert_allclose(got[keep], d["est"][keep], rtol=1e-9, atol=1e-10)
    if w.rotation and w.rot_den_type == 1 and nrotors(w) == 2:
        # the reference's running-sum conversion, rebuilt from the per-rotor
        # link means, equals its E_rot; the oracle's is the sum of the two
        m = rs_rotor_means(w, d["angles1"])
        ref_cum = rs_energy(w, rs_energy(w, m[0]) + m[1])
        assert ref_cum == pytest.approx(float(d["est"][2]), rel=1e-9)
        assert rot == pytest.approx(rs_energy(w, m[0]) + rs_energy(w, m[1]), rel=1e-9)


def test_densities_cycles_areas(case):
    """GetPotEnergy_Densities histograms, GetExchangeLength, GetAreaEstimators
    and GetAreaEstim3D (mc_estim.cc:500-687, 1233-1286, 1997-2594) of the
    final fixture path under the fixture's boson permutation."""
    name, w, d = case
    if "perm" not in d:
        pytest.skip("no bosons in this system")
    o = O.Oracle(w)
    o.set_state(d["coords1"], d["angles1"], d["perm"])
    v, g1, g2, g3 = o.densities()
    assert v == pytest.approx(float(d["dens_pot"]), rel=RTOL, abs=1e-12)
    np.testing.assert_array_equal(g1, dense_hist(d, "g1", g1.shape))
    np.testing.assert_array_equal(g2, dense_hist(d, "g2", g2.shape))
    np.testing.assert_array_equal(g3, dense_hist(d, "g3", g3.shape))
    assert g1.sum() + g2.sum() + g3.sum() > 0
    np.testing.assert_array_equal(o.exchange_lengths(len(d["ploops"])), d["ploops"])
    s_area, s_inert = area_scales(w, d["coords1"], d["masses"])
    if "area2d" in d:
        check_area(o.area_estimators(), d["area2d"], s_area, s_inert, False)
    for fr in (0, 1):
        check_area(o.area_estim3d(fr, d["masses"]), d["area3d"][fr], s_area, s_inert, True)
