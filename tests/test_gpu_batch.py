"""Replica batches (config-2 family): many independent systems in one
persistent launch.  A replica's moves and uniforms are those of a single
handle of the same system run with the replica's seed, so in FP64 the
batch must reproduce the single-system sampler path for path (the partner
sums are summed in another order, which changes action differences in the
last bits only; with no decision that close to its threshold the paths are
identical).  The warp count per CTA changes nothing.  Estimators of a batch
equal the single-system estimators of the same paths."""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu


def _small(n=5, seed=3):
    return W.config2(n=n, seed=seed, p_choices=(64, 128), n_he=(1, 6), t_range=(0.4, 1.5))


def test_batch_replicas_equal_single_systems_fp64():
    ws = _small()
    b = G.Batch(ws)
    b.set_shape(4)
    seed = 91
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
        rot = slice((w.natoms - 1) * w.nslices, (w.natoms - 1) * w.nslices + w.nrotslices)
        np.testing.assert_array_equal(ba[:, rot], an[:, rot])
        np.testing.assert_array_equal(bco[:, rot], co[:, rot])
        s.close()
    np.testing.assert_array_equal(btot, stot)
    np.testing.assert_array_equal(bacc, sacc)
    b.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_shape_does_not_change_the_paths(mixed):
    ws = _small(n=7, seed=8)
    states = []
    for warps, minb in ((2, 2), (8, 3)):
        b = G.Batch(ws, mixed=mixed)
        b.set_shape(warps, minb)
        b.run_passes(2, 5)
        b.synchronize()
        states.append([b.get_state(r)[0] for r in range(len(ws))])
        b.close()
    for x, y in zip(*states):
        np.testing.assert_array_equal(x, y)


def test_batch_estimators_equal_single_system_estimators():
    ws = _small(n=4, seed=12)
    b = G.Batch(ws, mixed=True)
    b.run_passes(3, 17)
    est = b.estimators()
    assert np.isfinite(est).all()
    for r, w in enumerate(ws):
        c, a, co, p = b.get_state(r)
        a_full = np.array(w.angles, copy=True)
        rot = slice((w.natoms - 1) * w.nslices, (w.natoms - 1) * w.nslices + w.nrotslices)
        a_full[:, rot] = a[:, rot]
        s = G.Sampler(w)
        s.set_state(c, a_full, p)
        e = s.estimators()
        np.testing.assert_allclose(est[r, :3], e[:3], rtol=1e-11, atol=1e-9)
        n = co[:, rot]
        np.testing.assert_allclose(est[r, 3], np.mean(n[2]), rtol=1e-12, atol=1e-14)
        s.close()
    b.close()


def test_batch_counts_the_reference_schedule_and_autotunes():
    ws = _small(n=6, seed=21)
    b = G.Batch(ws, mixed=True)
    shape, ms = b.autotune(33)
    assert shape[0] in (2, 4, 8) and shape[1] in (2, 3) and np.all(ms > 0)
    tot0, _ = b.counters()
    b.run_passes(1, 34)
    tot, acc = b.counters()
    d = tot - tot0
    P = np.array([w.nslices for w in ws]); N = np.array([w.types[0]["numb"] for w in ws])
    Q = np.array([w.nrotslices for w in ws])
    assert d[0] == N.sum() and d[1] == (N * P).sum()
    assert d[3] == len(ws) and d[4] == P.sum() and d[5] == (P * Q).sum()
    assert (acc <= tot).all()
    assert b.bead_moves_per_pass() == sum(w.bead_moves_per_pass() for w in ws)
    b.close()
