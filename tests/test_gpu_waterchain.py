"""The water-chain family (rotors on a chain, caleng between them, vcord to
the pH2 solvent, the analytic rattle-and-shake propagator): many replicas of
uneven rotor count, solvent count, slices and temperature in one persistent
launch.  In FP64 each replica must reproduce the single-system sampler run
with the replica's seed path for path, including replicas without solvent;
the batch estimators must equal the single-system estimators of the same
paths.  Per-move parity of this family with the reference is in the c4s
fixture (tests/test_gpu_parity.py)."""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu


def _family():
    tb = W.water_chain_tables(seed=5, grid3d=(30, 37, 19))
    spec = [(1, 0, 32, 0.7), (2, 3, 64, 1.6), (3, 1, 32, 1.1), (2, 0, 64, 0.5), (1, 2, 32, 2.0)]
    return [W.water_chain(nr, nh, P, P // 4, T, [9, k], tb, name="wc%d" % k) for k, (nr, nh, P, T) in
            enumerate(spec)]


def test_water_chain_replicas_equal_single_systems_fp64():
    ws = _family()
    b = G.Batch(ws)
    b.set_shape(4)
    seed = 41
    b.run_passes(2, seed)
    b.synchronize()
    btot, bacc = b.counters()
    stot = np.zeros(6); sacc = np.zeros(6)
    for r, w in enumerate(ws):
        s = G.Sampler(w)
        s.reset_counters()
        s.run_passes(2, G.Batch.replica_seed(seed, r))
        s.synchronize()
        t, a = s.counters()
        stot += t; sacc += a
        c, an, co, p = s.get_state()
        bc, ba, bco, bp = b.get_state(r)
        np.testing.assert_array_equal(bc, c)
        nh = w.types[0]["numb"]
        for k in range(w.types[1]["numb"]):
            rot = slice((nh + k) * w.nslices, (nh + k) * w.nslices + w.nrotslices)
            np.testing.assert_array_equal(ba[:, rot], an[:, rot])
        s.close()
    np.testing.assert_array_equal(btot, stot)
    np.testing.assert_array_equal(bacc, sacc)
    assert bacc[5] > 0 and bacc[4] > 0
    b.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_water_chain_batch_estimators_equal_single_systems(mixed):
    ws = _family()
    b = G.Batch(ws, mixed=mixed)
    b.run_passes(2, 7)
    est = b.estimators()
    assert np.isfinite(est).all()
    for r, w in enumerate(ws):
        c, a, co, p = b.get_state(r)
        a_full = np.array(w.angles, copy=True)
        nh = w.types[0]["numb"]
        for k in range(w.types[1]["numb"]):
            rot = slice((nh + k) * w.nslices, (nh + k) * w.nslices + w.nrotslices)
            a_full[:, rot] = a[:, rot]
        s = G.Sampler(w)
        s.set_state(c, a_full, p)
        e = s.estimators()
        np.testing.assert_allclose(est[r, :3], e[:3], rtol=1e-11, atol=1e-8)
        s.close()
    b.close()


def test_water_chain_counts_the_reference_schedule():
    ws = _family()
    b = G.Batch(ws, mixed=True)
    tot0, _ = b.counters()
    b.run_passes(1, 3)
    tot, acc = b.counters()
    d = tot - tot0
    P = np.array([w.nslices for w in ws]); Q = np.array([w.nrotslices for w in ws])
    NH = np.array([w.types[0]["numb"] for w in ws]); NR = np.array([w.types[1]["numb"] for w in ws])
    assert d[0] == NH.sum() and d[1] == (NH * P).sum()
    assert d[3] == NR.sum() and d[4] == (NR * P).sum() and d[5] == (NR * P * Q).sum()
    assert (acc <= tot).all()
    assert b.bead_moves_per_pass() == sum(w.bead_moves_per_pass() for w in ws)
    b.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_flat_half_sweeps_equal_the_persistent_pass(mixed):
    """Rotation mode 1 (one launch per half-sweep over all replicas, a warp
    per slice pair) makes the persistent pass's moves with its draws in its
    order per replica: the same paths and counters, bit for bit, for the
    water chains and for the linear-rotor family."""
    for ws in (_family(), W.config2(n=5, seed=3, p_choices=(64, 128), n_he=(1, 6), t_range=(0.4, 1.5))):
        out = []
        for mode in (0, 1):
            b = G.Batch(ws, mixed=mixed)
            b.set_shape(4)
            b.set_rotation_mode(mode)
            b.run_passes(2, 19)
            b.synchronize()
            out.append(([b.get_state(r)[:2] for r in range(len(ws))], b.counters()))
            b.close()
        for m in (1,):
            for (c0, a0), (c1, a1) in zip(out[0][0], out[m][0]):
                np.testing.assert_array_equal(c0, c1)
                np.testing.assert_array_equal(a0, a1)
            np.testing.assert_array_equal(out[0][1][0], out[m][1][0])
            np.testing.assert_array_equal(out[0][1][1], out[m][1][1])


def test_fp32_batch_samples_the_fp64_distribution():
    """The FP32 path of the water-chain batch (float pair terms and densities;
    each accepted rotor move updates the other rotors' cached potentials at
    its slice by the change of their pair term instead of invalidating them)
    samples the FP64 path's distribution.  K identical replicas of a small
    chain (3 waters on the 3 A chain + 2 pH2, P = 64, Q = 16, 5 K), brought to
    equilibrium by EQ0 FP64 passes; each precision starts from those states,
    makes EQ passes of its own, then samples the estimators after every pass.
    The error of a mean is the spread of the K chain means over sqrt(K).
    Criterion: E_kin, E_pot and E_rot each within 3 combined standard errors
    and at most one of the three beyond 2."""
    K, EQ0, EQ, NS = 128, 200, 30, 100
    tb = W.water_chain_tables(seed=5, grid3d=(30, 37, 19))
    w = W.water_chain(3, 2, 64, 16, 5.0, [9, 7], tb, name="wc-stat")
    b = G.Batch([w] * K)
    b.set_rotation_mode(1)
    b.run_passes(EQ0, 41)
    start = [b.get_state(r) for r in range(K)]
    b.close()
    res = {}
    for mixed, seed in ((False, 1000), (True, 2000)):
        b = G.Batch([w] * K, mixed=mixed)
        b.set_rotation_mode(1)
        for r, (c, a, _, p) in enumerate(start):
            b.set_state(r, c, a, p)
        b.run_passes(EQ, seed)
        acc = np.zeros((K, 3))
        for k in range(NS):
            b.run_passes(1, seed)
            acc += b.estimators()[:, :3]
        b.close()
        means = acc / NS
        res[mixed] = (means.mean(0), means.std(0, ddof=1) / np.sqrt(K))
    (m0, e0), (m1, e1) = res[False], res[True]
    z = (m1 - m0) / np.hypot(e0, e1)
    print("E_kin, E_pot, E_rot FP64", m0, "+-", e0, "FP32 path", m1, "+-", e1, "z", z)
    assert np.all(np.isfinite(z)) and np.all(np.abs(z) <= 3.0), z
    assert int(np.sum(np.abs(z) > 2.0)) <= 1, z
