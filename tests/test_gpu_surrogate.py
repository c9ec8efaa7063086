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


def test_delayed_acceptance_samples_the_exact_distribution():
    """Plain and surrogate-screened chains from the same start: the mean
    dimer energy over the run agrees within the spread of block means."""
    w, s = _dimer()
    s.da_sweeps(50, seed=2)
    x, e = _collect(s, 80, 2, seed=300)
    mu, sd = float(e.mean()), float(e.std())
    m = G.Mlp()
    rng = np.random.default_rng(1)
    m.set_weights(rng.normal(0, 1 / np.sqrt(6), (6, 256)), np.zeros(256), rng.normal(0, 1 / 16, (256, 256)),
                  np.zeros(256), rng.normal(0, 1 / 16, (256, 256)), np.zeros(256), rng.normal(0, 1 / 16, 256), 0.0)
    m.train(x, (e - mu) / sd, epochs=15, batch=1024, lr=1e-3, seed=4)
    c0, a0, co0, p0 = s.get_state()
    means = {}
    for use in (False, True):
        sx = G.Sampler(w)
        sx.set_state(c0, a0, p0)
        blocks = []
        for b in range(12):
            sx.da_sweeps(10, seed=1000 + b, mlp=m if use else None, escale=sd)
            blocks.append(float(sx.da_samples()[1].mean()))
        means[use] = (np.mean(blocks[2:]), np.std(blocks[2:]) / np.sqrt(len(blocks) - 2))
        sx.close()
    (m0, e0), (m1, e1) = means[False], means[True]
    assert abs(m0 - m1) <= 5 * np.hypot(e0, e1) + 0.05 * sd, (means, sd)
    s.close()
    m.close()
