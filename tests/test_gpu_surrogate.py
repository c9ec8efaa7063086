"""The surrogate in the sampler (two-stage delayed acceptance) on a small water
dimer (P = 128, Q = 64): training data emitted by the sampler, the MLP
trained on the GPU by its tensor-core kernels, and the two-stage
delayed-acceptance rotational move whose second stage uses the exact caleng
potential."""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu


def _dimer():
    w = W.config3(nslices=128, nrotslices=64, griddens=(37, 73, 73))
    s = G.Sampler(w)
    return w, s


def _collect(s, ncalls, sweeps_between, seed):
    feats, ens = [], []
    for k in range(ncalls):
        s.da_sweeps(sweeps_between, seed + k)
        f, e = s.da_samples()
        feats.append(f)
        ens.append(e)
    return np.concatenate(feats), np.concatenate(ens)


def test_plain_sweeps_and_samples():
    w, s = _dimer()
    st = s.da_sweeps(20, seed=1)
    assert st[0] == 20 * w.nrotslices * 2 and st[1] == st[0] and st[3] == st[0]
    assert 0 < st[2] < st[0]
    f, e = s.da_samples()
    assert f.shape == (w.nslices, 6) and np.isfinite(f).all() and np.isfinite(e).all()
    assert np.all(f[:, 0] > -6.0)             # r > 0
    np.testing.assert_allclose(np.linalg.norm(f[:, 1:4], axis=1), 1.0, atol=1e-5)   # a unit vector on three axes
    s.close()


def test_surrogate_delayed_acceptance():
    w, s = _dimer()
    s.da_sweeps(50, seed=2)                       # leave the start
    x, e = _collect(s, 120, 2, seed=100)
    mu, sd = float(e.mean()), float(e.std())
    m = G.Mlp()
    rng = np.random.default_rng(0)
    m.set_weights(rng.normal(0, 1 / np.sqrt(6), (6, 256)), np.zeros(256), rng.normal(0, 1 / 16, (256, 256)),
                  np.zeros(256), rng.normal(0, 1 / 16, (256, 256)), np.zeros(256), rng.normal(0, 1 / 16, 256), 0.0)
    ntr = (len(x) // 1024 - 2) * 1024
    losses = m.train(x[:ntr], (e[:ntr] - mu) / sd, epochs=25, batch=1024, lr=1e-3, seed=3)
    assert losses[-1] < losses[0]
    pred = m.forward(x[ntr:]) * sd + mu
    rms = float(np.sqrt(np.mean((pred - e[ntr:]) ** 2)))
    assert rms < 0.5 * sd, (rms, sd)              # the network learned the dimer energy
    # delayed acceptance: exact differences only behind the first stage
    st = s.da_sweeps(40, seed=7, mlp=m, escale=sd)
    assert st[0] == 40 * w.nrotslices * 2
    assert st[3] == st[1] and st[2] <= st[1] <= st[0] and st[2] > 0
    c, a, co, p = s.get_state()
    assert np.isfinite(c).all() and np.isfinite(a).all()
    s.close()
    m.close()


def test_screen_is_exact_and_reports_its_cost():
    """The screened chain samples the exact distribution; what the screen
    saves is measured and reported.

    K identical small dimers (P = 64, Q = 32) in one batch, each replica an
    independent chain of rotational sweeps with its own seed.  The replicas
    are first brought to equilibrium by EQ0 plain sweeps; both arms start
    from those states, make EQ sweeps of their own, then sample the
    estimators every EVERY sweeps.  The error of an arm's mean is the spread
    of the K chain means over sqrt(K).  Exactness: E_pot (the dimer energy
    the surrogate screens) and E_rot agree between the plain and the screened
    arm within 2 combined standard errors.  The screen stops a share of the
    proposals before the exact difference (asserted: fewer exact evaluations
    than proposals).  Cost at equal error: the exact evaluations an arm needs
    for a given error scale as (exact evaluations per sweep) x SE^2 at equal
    sweeps; the ratio screened / plain is printed.  It is not asserted below
    1: with the six dimer features (which leave the second top's turn about
    its own axis out) the surrogate's error lowers the acceptance (0.41 of
    the proposals against 0.55) nearly as much as the screen saves (0.67
    exact evaluations per proposal), and two runs measured 1.18 and 0.79 --
    no saving distinguishable from the ratio's own scatter at K = 256.  The
    benchmark reports the same crossover in wall time."""
    K, EQ0, EQ, NS, EVERY = 256, 3000, 200, 100, 5
    w = W.config3(seed=40, nslices=64, nrotslices=32, griddens=(19, 37, 37), levels=4)
    s = G.Sampler(w)
    s.da_sweeps(50, seed=2)
    x, e = _collect(s, 1000, 2, seed=500)
    s.close()
    mu, sd = float(e.mean()), float(e.std())
    m = G.Mlp()
    rng = np.random.default_rng(1)
    m.set_weights(rng.normal(0, 1 / np.sqrt(6), (6, 256)), np.zeros(256), rng.normal(0, 1 / 16, (256, 256)),
                  np.zeros(256), rng.normal(0, 1 / 16, (256, 256)), np.zeros(256), rng.normal(0, 1 / 16, 256), 0.0)
    m.train(x, (e - mu) / sd, epochs=25, batch=1024, lr=1e-3, seed=4)
    b = G.Batch([w] * K)
    b.da_sweeps(EQ0, 777)
    start = [b.get_state(r) for r in range(K)]
    b.close()
    res = {}
    for arm, mlp, base in (("plain", None, 10000), ("screened", m, 20000)):
        b = G.Batch([w] * K)
        for r, (c, a, _, p) in enumerate(start):
            b.set_state(r, c, a, p)
        b.da_sweeps(EQ, base, mlp=mlp, escale=sd)
        acc = np.zeros((K, 2))
        st = np.zeros(4)
        for k in range(NS):
            st += b.da_sweeps(EVERY, base + 1, mlp=mlp, escale=sd)     # the pass counters key each call's draws
            acc += b.estimators()[:, 1:3]
        b.close()
        means = acc / NS
        res[arm] = (means.mean(0), means.std(0, ddof=1) / np.sqrt(K), st)
    (m0, e0, st0), (m1, e1, st1) = res["plain"], res["screened"]
    z = (m1 - m0) / np.hypot(e0, e1)
    cost = (st1[3] * e1[0] ** 2) / (st0[3] * e0[0] ** 2)
    print("E_pot, E_rot plain", m0, "+-", e0, "screened", m1, "+-", e1, "z", z)
    print("exact evaluations per proposal: plain %.3f screened %.3f; per accepted move: plain %.3f screened %.3f; "
          "exact evaluations for equal SE of E_pot, screened / plain: %.3f"
          % (st0[3] / st0[0], st1[3] / st1[0], st0[3] / st0[2], st1[3] / st1[2], cost))
    assert st0[3] == st0[0] and st0[0] == st1[0] == NS * EVERY * K * w.nrotslices * 2
    assert np.all(np.abs(z) <= 2.0), z
    assert st1[3] < st1[0]
    assert np.isfinite(cost) and cost > 0.0
    m.close()
