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


@pytest.mark.parametrize("surrogate", [False, True])
def test_batch_da_replicas_equal_single_systems(surrogate):
    ws = _dimers()
    m = _mlp() if surrogate else None
    b = G.Batch(ws)
    seed = 12
    st = b.da_sweeps(6, seed, mlp=m, escale=300.0)
    assert st[0] == 6 * sum(w.nrotslices * 2 for w in ws)
    sst = np.zeros(4)
    for r, w in enumerate(ws):
        s = G.Sampler(w)
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
