"""The synthetic workloads (moribs-pimc_gb300/workloads.py) have the shapes
the benchmark's five configurations name: species and counts, rotational
constants, temperatures, translational and rotational slices, bisection
levels, table sizes, and for the replica families the ranges each replica is
drawn from.  No GPU; the config-2 and config-4 families are built at their
full replica counts."""
import numpy as np

import workloads as W


def _types(w):
    return {t["name"]: t for t in w.types}


def test_config0_linear_rotor_and_helium():
    w = W.config0()
    t = _types(w)
    assert t["CO2"]["numb"] == 1 and t["CO2"]["molecule"] == 1
    assert t["He4"]["numb"] == 8 and t["He4"]["molecule"] == 0 and t["He4"]["stat"] == 1
    assert (w.nslices, w.nrotslices, w.temperature) == (512, 128, 0.37)
    assert all(tt["levels"] == 3 for tt in w.types)
    g = np.asarray(w.tables["grid1d"])
    assert len(g) == 512 and g[0] == 1.0 and g[-1] == 30.0          # He-He table on 1-30 A, 512 points


def test_config1_asymmetric_top_and_para_hydrogen():
    w = W.config1()
    t = _types(w)
    assert t["SO2"]["numb"] == 1 and t["SO2"]["molecule"] == 2
    assert t["H2"]["numb"] == 64 and t["H2"]["molecule"] == 0
    assert tuple(w.rot_abc) == (2.03, 0.344, 0.293)
    assert (w.nslices, w.nrotslices, w.temperature) == (1024, 256, 0.37)
    assert len(w.tables["grid1d"]) == 1024                             # pH2-pH2 table, 1024 points
    assert (w.tables["rgrd"], w.tables["thgrd"], w.tables["chgrd"]) == (200, 60, 60)
    assert np.asarray(w.tables["rhoprp"]).shape == (61, 121, 121)
    assert w.bead_moves_per_pass() == 64 * 1024 * 7 + 64 * 1024 + 1 * 1024 * 7 + 1024 + 1024 * 256


def test_config2_family_ranges():
    ws = W.config2()
    assert len(ws) == 4096
    n_he = np.array([_types(w)["He4"]["numb"] for w in ws])
    P = np.array([w.nslices for w in ws])
    Q = np.array([w.nrotslices for w in ws])
    T = np.array([w.temperature for w in ws])
    assert n_he.min() >= 1 and n_he.max() <= 64 and len(set(n_he)) > 32
    assert set(P) == {64, 128, 256, 512} and (Q * 4 == P).all()
    assert T.min() >= 0.3 and T.max() <= 2.0


def test_config3_water_dimer():
    w = W.config3()
    t = _types(w)
    assert t["H2O"]["numb"] == 2 and t["H2O"]["molecule"] == 2
    assert tuple(w.rot_abc) == (27.9, 14.5, 9.3)
    assert (w.nslices, w.nrotslices, w.temperature) == (4096, 2048, 0.74)


def test_config4_family_ranges():
    ws = W.config4()
    assert len(ws) == 512
    nr = np.array([_types(w)["H2O"]["numb"] for w in ws])
    nh = np.array([_types(w)["H2"]["numb"] for w in ws])
    P = np.array([w.nslices for w in ws])
    Q = np.array([w.nrotslices for w in ws])
    T = np.array([w.temperature for w in ws])
    assert nr.min() >= 1 and nr.max() <= 8 and set(nr) == set(range(1, 9))
    assert nh.min() >= 0 and nh.max() <= 32 and (nh == 0).any()
    assert set(P) <= {512, 1024, 2048} and (Q * 4 == P).all() and Q.min() >= 128 and Q.max() <= 512
    assert T.min() >= 0.5 and T.max() <= 2.0
    # the waters on a line 3 A apart (x), at the start of every replica's path
    w = next(w for w in ws if _types(w)["H2O"]["numb"] >= 3)
    nh0 = _types(w)["H2"]["numb"]
    x = np.array([w.coords[0, (nh0 + k) * w.nslices] for k in range(_types(w)["H2O"]["numb"])])
    np.testing.assert_allclose(np.diff(x), 3.0, atol=0.1)
