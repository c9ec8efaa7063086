"""GPU parity: the sm_103a kernels (through the C ABI) against the oracle and
the fixtures generated from the reference's own C++.

FP64 tolerance: 1e-10 relative.  An action difference is a difference of
nearly equal sums, so its error bound is 1e-10 of the magnitude of the terms
it is made of (|E_new| + |E_old|), not of the difference itself."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W
from _common import golden, golden_cases, rot_est_from_reference, split_streams

pytestmark = pytest.mark.gpu
RTOL = 1e-10


@pytest.fixture(scope="module", params=golden_cases())
def case(request):
    w, d, M = golden(request.param)
    return request.param, w, d


def _close(a, b, scale=None, rtol=RTOL):
    a, b = np.asarray(a, float), np.asarray(b, float)
    s = np.maximum(np.abs(b), 1.0) if scale is None else np.maximum(np.asarray(scale, float), 1e-300)
    bad = np.abs(a - b) > rtol * s
    assert not bad.any(), "max rel err %g at %s: %s vs %s" % (
        np.max(np.abs(a - b) / s), np.argwhere(bad)[:3].ravel(), a[bad][:3], b[bad][:3])


def test_pot_energy_matches_reference_fixture(case):
    name, w, d = case
    s = G.Sampler(w)
    s.set_state(d["coords0"], d["angles0"], w.pindex)
    P = w.nslices
    a0, it, xyz, ref = [], [], [], []
    for a in range(w.natoms):
        for j, t in enumerate(d["slices"]):
            for k, arr in enumerate((d["coords0"], d["pos"])):
                a0.append(a); it.append(t); xyz.append(arr[:, a * P + t]); ref.append(d["e_slice"][a, j, k])
    got = s.pot_energy(a0, it, np.array(xyz))
    _close(got, ref)
    s.close()


def test_rot_energy_matches_reference_fixture(case):
    name, w, d = case
    if not w.rotation:
        pytest.skip("no rotational slices in this system")
    s = G.Sampler(w)
    s.set_state(d["coords0"], d["angles0"], w.pindex)
    rtype = [i for i, t in enumerate(w.types) if t["molecule"] != 0][0]
    roff = sum(t["numb"] for t in w.types[:rtype])
    linear = w.types[rtype]["molecule"] == 1
    rot, its, v3, ref = [], [], [], []
    for k in range(d["eul"].shape[0]):
        e = d["eul"][k]
        for j, t in enumerate(d["slices"]):
            rot.append(roff); its.append(t); ref.append(d["e_rot"][k, j])
            if linear:
                v3.append([np.sin(e[1]) * np.cos(e[0]), np.sin(e[1]) * np.sin(e[0]), np.cos(e[1])])
            else:
                v3.append(e)
    got = s.pot_rot_energy(rot, its, np.array(v3))
    _close(got, ref)
    s.close()


def test_move_sequence_matches_oracle_and_reference(case):
    """Every reference call of the fixture's sequence, replayed on the GPU
    and on the oracle in lockstep: identical random-number consumption,
    identical accept decisions, action differences to FP64 parity, and the
    final path equal to the reference's.

    Tolerances follow from the 1e-10 bound on the energy terms: a bisection
    level difference sums up to 2M slice energies times tau*M/2; a centroid
    dV sums 2P; a rotational ratio carries exp(-tau dV) with dV from 2R
    slice sums, so its relative error is tau * 2R * |E| * 1e-10."""
    name, w, d = case
    s = G.Sampler(w)
    o = O.Oracle(w)
    st = split_streams(d)
    tau = 1.0 / (w.temperature * w.nslices)
    emax = float(np.max(np.abs(d["e_slice"])))
    erot = float(np.max(np.abs(d["e_rot"])))
    R = w.nslices // w.nrotslices
    ib = im = ir = 0
    for kind, typ, t in d["seq"]:
        typ, t = int(typ), int(t)
        if kind == 0:
            g, u3 = st["gauss"][ib], st["u3"][ib]; ib += 1
            rs, ds, lv, cons = s.bisection_move(typ, t, g, u3)
            _, ods, olv, ocons = o.bisection_move(typ, t, g, u3)
            assert rs == 0
            assert cons == ocons
            np.testing.assert_array_equal(lv, olv)
            mask = np.arange(ds.shape[1])[None, :] <= np.minimum(lv, ds.shape[1] - 1)[:, None]
            M = 1 << w.types[typ]["levels"]
            _close(ds[mask], ods[mask], scale=np.maximum(np.abs(ods[mask]), tau * M * M * emax))
        elif kind == 1:
            u1, u2 = st["u1"][im], st["u2"][im]; im += 1
            rs, dv, acc, cons = s.molecular_move(typ, u1, u2)
            _, odv, oacc, ocons = o.molecular_move(typ, u1, u2)
            assert rs == 0
            assert cons == ocons
            np.testing.assert_array_equal(acc, oacc)
            _close(dv, odv, scale=np.maximum(np.abs(odv), 2 * w.nslices * emax))
        else:
            ur = st["urot"][ir]; ir += 1
            rs, rd, acc = s.rotations(ur)
            _, ord_, oacc, opos = o.rotations(typ, ur)
            assert rs == 0
            np.testing.assert_array_equal(acc, oacc)
            _close(rd, ord_, scale=np.maximum(np.abs(ord_), 1.0) * max(1.0, tau * 2 * R * erot))
    c, a, co, _ = s.get_state()
    _close(c, d["coords1"])
    _close(a, d["angles1"])
    _close(co, d["cosine1"])
    tot, acc = s.counters()
    np.testing.assert_array_equal(tot[:len(d["total"])], d["total"])
    np.testing.assert_array_equal(acc[:len(d["accep"])], d["accep"])
    s.close()


def test_estimators_match_reference_fixture(case):
    name, w, d = case
    s = G.Sampler(w)
    s.set_state(d["coords1"], d["angles1"], w.pindex)
    est = s.estimators()
    o = O.Oracle(w)
    o.set_state(d["coords1"], d["angles1"], w.pindex)
    # the reference's values where its GetRotE3D computes what it intends,
    # else the oracle's (each rotor at its own offset, converted once)
    erot_ok, sq_ok = rot_est_from_reference(w)
    want = np.array(d["est"], dtype=np.float64)
    if w.rotation and not (erot_ok and sq_ok):
        rot, esq, ets = o.rot_energy(True)
        if not erot_ok:
            want[2] = rot
        if not sq_ok:
            want[3], want[4] = esq, ets
    _close(est, want, scale=np.maximum(np.abs(want), 1.0))
    if w.rotation and any(t["molecule"] != 0 for t in w.types):
        _close(s.rcf(), o.rcf())
    s.close()


def test_config1_full_size_energies():
    """config 1 at its full size (P=1024, 64 pH2, 200x60x60 potential,
    61x121x121 density): PotEnergy and PotRotE3D queries against the oracle."""
    w = W.config1()
    s = G.Sampler(w)
    o = O.Oracle(w)
    rng = np.random.default_rng(9)
    P = w.nslices
    a0 = rng.integers(0, w.natoms, 200)
    it = rng.integers(0, P, 200)
    xyz = np.array([w.coords[:, a * P + t] + rng.normal(0, 0.2, 3) for a, t in zip(a0, it)])
    got = s.pot_energy(a0, it, xyz)
    ref = []
    for a, t, x in zip(a0, it, xyz):
        pos = w.coords.copy()
        pos[:, a * P + t] = x
        ref.append(o.pot_energy_slice(int(a), pos, int(t)))
    _close(got, ref)
    eul = np.column_stack([rng.uniform(0, 2 * np.pi, 64), np.arccos(rng.uniform(-1, 1, 64)), rng.uniform(0, 2 * np.pi, 64)])
    its = rng.integers(0, P, 64)
    got = s.pot_rot_energy(np.full(64, 64), its, eul)
    ref = [o.pot_rot_e3d(64, e, int(t)) for e, t in zip(eul, its)]
    _close(got, ref)
    s.close()


def test_config0_full_size_replay_moves():
    """config 0 at full size (P=512, Q=128, 8 He + CO2): bisection at several
    start slices and one full rotational sweep, in lockstep with the oracle."""
    w = W.config0()
    s = G.Sampler(w)
    o = O.Oracle(w)
    rng = np.random.default_rng(4)
    for t in (0, 100, 509):
        for typ in (0, 1):
            g = rng.normal(size=3 * 8 * 9)
            u3 = rng.uniform(size=30)
            rs, ds, lv, cons = s.bisection_move(typ, t, g, u3)
            _, ods, olv, ocons = o.bisection_move(typ, t, g, u3)
            assert rs == 0 and cons == ocons
            np.testing.assert_array_equal(lv, olv)
    c0, a0, co0, _ = o.get_state()
    erot = max(abs(o.pot_rot_energy(8, co0, t)) for t in range(0, w.nslices, 37))
    tau = 1.0 / (w.temperature * w.nslices)
    ur = rng.uniform(size=3 * w.nrotslices)
    rs, rd, acc = s.rotations(ur)
    _, ord_, oacc, _ = o.rotations(1, ur)
    assert rs == 0
    np.testing.assert_array_equal(acc, oacc)
    _close(rd, ord_, scale=np.maximum(np.abs(ord_), 1.0) * max(1.0, tau * 8 * erot))
    c, a, co, _ = s.get_state()
    c2, a2, co2, _ = o.get_state()
    _close(c, c2)
    _close(a, a2)
    s.close()


def test_production_pass_schedules_the_reference_move_counts(case):
    """One production pass performs exactly the reference schedule's moves:
    per type N centroid moves and N*P bisections, P*Q rotation attempts per
    rotor (mc_main.cc:348-381); the path stays finite."""
    name, w, d = case
    s = G.Sampler(w)
    s.reset_counters()
    s.run_passes(2, seed=123)
    s.synchronize()
    tot, acc = s.counters()
    P = w.nslices
    for i, t in enumerate(w.types):
        assert tot[3 * i + 0] == 2 * t["numb"]
        assert tot[3 * i + 1] == 2 * t["numb"] * P
        if t["molecule"] != 0 and w.rotation:
            assert tot[3 * i + 2] == 2 * t["numb"] * P * w.nrotslices
    assert (acc <= tot).all()
    c, a, co, _ = s.get_state()
    assert np.isfinite(c).all() and np.isfinite(a).all()
    est = s.estimators()
    assert np.isfinite(est).all()
    s.close()


def test_vcord_at_grid_nodes():
    """vcalc's one-sided differences jump across a grid node (vcalc.f:31-60),
    so at a node the reference's value depends on the last bit of acos/atan
    (CUDA's and glibc's may differ by an ulp) and of the divisions by the
    steps (vcord.f:88-91, vcalc.f:21-23), which the GPU repeats there.  Each
    slice puts one pH2 bead where the body-frame (r, theta, chi) of the
    rotor's identity frame is a node of the c1s grid (r = rvmin + n rstep in
    bohr, theta = k dth, chi = m dch); the GPU's rotor-pH2 sum must equal the
    oracle's on one of the two sides of the node in each coordinate (the
    node approached from r, theta, chi -/+ 1e-12), to 1e-10."""
    w, d, _ = golden("c1s")
    tb = w.tables
    P, na = w.nslices, w.natoms
    bo2ang = 0.529177249
    rstep = (tb["rvmax"] - tb["rvmin"]) / (tb["rgrd"] - 1)
    dth = 180.0 / (tb["thgrd"] - 1)
    dch = float(tb["chi_fold_deg"]) / (tb["chgrd"] - 1)
    rng = np.random.default_rng(17)
    roff = na - 1                       # the rotor is the last atom
    nodes = []
    for it in range(P):
        n = int(rng.integers(2, tb["rgrd"] - 2))
        k = int(rng.integers(1, tb["thgrd"] - 1))
        m = int(rng.integers(1, tb["chgrd"] - 1))
        nodes.append(((tb["rvmin"] + n * rstep) * bo2ang, np.radians(k * dth), np.radians(m * dch)))

    def place(dr, dt, dc):
        c = np.array(d["coords0"], copy=True)
        for it, (rho, th, ch) in enumerate(nodes):
            rho, th, ch = rho + dr, th + dt, ch + dc
            rc = c[:, roff * P + it]
            c[:, it] = rc + rho * np.array([np.sin(th) * np.cos(ch), np.sin(th) * np.sin(ch), np.cos(th)])
        return c
    eul = np.zeros(3)
    s = G.Sampler(w)
    s.set_state(place(0.0, 0.0, 0.0), d["angles0"], w.pindex)
    got = s.pot_rot_energy([roff] * P, list(range(P)), np.tile(eul, (P, 1)))
    s.close()
    o = O.Oracle(w)
    sides = []
    eps = 1e-12
    for dr in (-eps, eps):
        for dt in (-eps, eps):
            for dc in (-eps, eps):
                o.set_state(place(dr, dt, dc), d["angles0"], w.pindex)
                sides.append([o.pot_rot_e3d(roff, eul, it) for it in range(P)])
    sides = np.array(sides)                                   # [8, P]
    err = np.min(np.abs(sides - got[None, :]), axis=0) / np.maximum(np.abs(sides).max(axis=0), 1.0)
    assert np.all(err <= 1e-10), (err, got, sides)
    # the nodes are real discontinuities: somewhere the two sides differ
    assert np.max(np.ptp(sides, axis=0)) > 1e-6


