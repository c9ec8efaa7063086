"""Delayed acceptance over a batch of water dimers (pimc_batch_da_sweeps,
pimc_batch_da_passes): one proposal launch, one surrogate launch and one
decision launch per sub-phase for all replicas.  Replica r must make
exactly the moves of a single handle swept with the replica's seed, with and
without the surrogate; the passes must count the reference schedule's moves."""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu


def _dimers(n=3):
    return [W.config3(seed=40 + k, nslices=64, nrotslices=32, griddens=(19, 37, 37), levels=4) for k in range(n)]


def _mlp(seed=3):
    rng = np.random.default_rng(seed)
    m = G.Mlp(0)
    m.set_weights(rng.normal(0, 1 / np.sqrt(6), (6, 256)), rng.normal(0, 0.1, 256), rng.normal(0, 1 / 16, (256, 256)),
                  rng.normal(0, 0.1, 256), rng.normal(0, 1 / 16, (256, 256)), rng.normal(0, 0.1, 256),
                  rng.normal(0, 1 / 16, 256), 0.0)
    return m


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("surrogate", [False, True])
def test_batch_da_replicas_equal_single_systems(surrogate, mixed):
    ws = _dimers()
    m = _mlp() if surrogate else None
    b = G.Batch(ws, mixed=mixed)
    seed = 12
    st = b.da_sweeps(6, seed, mlp=m, escale=300.0)
    assert st[0] == 6 * sum(w.nrotslices * 2 for w in ws)
    sst = np.zeros(4)
    for r, w in enumerate(ws):
        s = G.Sampler(w, mixed=mixed)
        sst += s.da_sweeps(6, G.Batch.replica_seed(seed, r), mlp=m, escale=300.0)
        _, a, co, _ = s.get_state()
        _, ba, bco, _ = b.get_state(r)
        for k in range(2):
            rot = slice(k * w.nslices, k * w.nslices + w.nrotslices)
            np.testing.assert_array_equal(ba[:, rot], a[:, rot])
        s.close()
    np.testing.assert_array_equal(st, sst)
    if surrogate:
        assert st[3] < st[0]                 # some proposals stopped at the first stage
        m.close()
    b.close()


def test_batch_da_passes_count_the_schedule():
    ws = _dimers(2)
    b = G.Batch(ws)
    tot0, _ = b.counters()
    st = b.da_passes(2, 5)
    tot, acc = b.counters()
    d = tot - tot0
    P, Q = ws[0].nslices, ws[0].nrotslices
    n = len(ws)
    assert d[0] == 2 * 2 * n and d[1] == 2 * 2 * n * P      # centroid, bisection of the two tops
    assert d[2] == 2 * 2 * n * P * Q                         # P sweeps of 2 x Q rotational slices per pass
    assert st[0] == 2 * 2 * n * P * Q and 0 < st[2] <= st[0]
    e = b.estimators()
    assert np.isfinite(e).all()
    b.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_da_passes_sample_the_standard_distribution(mixed):
    """Passes whose rotational sweeps are made by the delayed-acceptance
    kernels without a screen (plain Metropolis, the link cache of the
    tabulated densities kept by those kernels) and the batch's standard
    passes sample the same distribution, in both precisions (on the FP32
    path both arms make the FP32 path's moves).  K identical dimers of the
    statistics tests' config-3 shape (5 K, P = 64, Q = 32, bisection levels 2,
    centroid step 0.02 A), brought to equilibrium by EQ0 standard passes; each
    arm starts from those states, makes EQ passes of its own, then samples
    the estimators after every pass.  The error of an arm's mean is the
    spread of the K chain means over sqrt(K).  Criterion: E_kin, E_pot and
    E_rot each within 3 combined standard errors and at most one of the three
    beyond 2."""
    K, EQ0, EQ, NS = 256, 300, 30, 100
    w = W.config3(seed=7, nslices=64, nrotslices=32, griddens=(19, 37, 37), levels=2)
    w.types[0]["mcstep"] = 0.02
    w.temperature = 5.0
    b = G.Batch([w] * K, mixed=mixed)
    b.run_passes(EQ0, 31)
    start = [b.get_state(r) for r in range(K)]
    b.close()
    res = {}
    for arm, seed in (("standard", 1000), ("delayed", 2000)):
        b = G.Batch([w] * K, mixed=mixed)
        for r, (c, a, _, p) in enumerate(start):
            b.set_state(r, c, a, p)
        run = b.run_passes if arm == "standard" else b.da_passes
        run(EQ, seed)
        acc = np.zeros((K, 3))
        for k in range(NS):
            run(1, seed)                     # the pass counters key each pass's draws
            acc += b.estimators()[:, :3]
        b.close()
        means = acc / NS
        res[arm] = (means.mean(0), means.std(0, ddof=1) / np.sqrt(K))
    (m0, e0), (m1, e1) = res["standard"], res["delayed"]
    z = (m1 - m0) / np.hypot(e0, e1)
    print("E_kin, E_pot, E_rot standard", m0, "+-", e0, "delayed-acceptance kernels", m1, "+-", e1, "z", z)
    assert np.all(np.isfinite(z)) and np.all(np.abs(z) <= 3.0), z
    assert int(np.sum(np.abs(z) > 2.0)) <= 1, z
