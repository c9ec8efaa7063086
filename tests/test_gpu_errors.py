"""Error paths of the C ABI that must leave the handle usable.

* A PIndex that is not a permutation of the boson type's own atoms is
  rejected on the host (PIMC_ERR_BAD_ARG) before anything reaches the
  device: the exchange moves and estimators walk its cycles
  (mc_piqmc.cc:129-138, mc_estim.cc:2008-2013).
* A persistent rotational sweep whose wait for a neighbouring slice runs
  out sets the abort word and ends; the next synchronising call returns
  PIMC_ERR_TIMEOUT and the handle then runs normally.  The test makes the
  wait run out by setting its limit to zero (PIMC_OPT_WAIT_NS): a slice that
  does not find both neighbours done at its first poll gives up.  No kernel
  is broken and nothing waits longer than the limit.
"""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu

ERR_BAD_ARG = 1
ERR_TIMEOUT = 5
OPT_WAIT_NS = 3


def _bad(fn):
    with pytest.raises(G.PimcError) as ei:
        fn()
    assert ei.value.code == ERR_BAD_ARG
    return ei.value.code


def test_bad_permutation_rejected():
    w = W.config0(seed=3, nslices=64, nrotslices=16, n_he=4, r2d_step=0.05, c2d_step=0.04)
    s = G.Sampler(w, device=0)
    c0, a0, _, p0 = s.get_state()
    na = w.natoms
    ident = np.arange(na, dtype=np.int32)
    # not a bijection (walks that never close)
    p = ident.copy(); p[0] = 1; p[1] = 1
    _bad(lambda: s.set_state(c0, a0, p))
    # a cycle leaving the boson type (He atoms are 0..3, the rotor is atom 4)
    p = ident.copy(); p[3] = 4; p[4] = 3
    _bad(lambda: s.set_state(c0, a0, p))
    # out of range
    p = ident.copy(); p[2] = na
    _bad(lambda: s.set_state(c0, a0, p))
    # nothing changed: the path and permutation are the ones set before
    c1, a1, _, p1 = s.get_state()
    assert np.array_equal(c1, c0) and np.array_equal(a1, a0) and np.array_equal(p1, p0)
    # a valid 3-cycle of the bosons is accepted and the exchange move runs
    p = ident.copy(); p[0], p[1], p[2] = 1, 2, 0
    s.set_state(c0, a0, p)
    rng = np.random.default_rng(1)
    s.molecular_move_exchange(0, rng.uniform(size=64), rng.uniform(size=64))
    assert np.array_equal(s.get_state()[3], p)
    s.close()


def test_batch_bad_permutation_rejected():
    ws = W.config2(n=2, seed=11)
    b = G.Batch(ws, device=0, mixed=False)
    c, a, _, p = b.get_state(0)
    p = np.array(p, dtype=np.int32)
    q = p.copy(); q[0] = q[1]
    _bad(lambda: b.set_state(0, c, a, q))
    b.set_state(0, c, a, p)
    b.run_passes(1, 5)
    b.synchronize()
    b.close()


def test_sweep_wait_timeout_recovers():
    w = W.config0(seed=5, nslices=256, nrotslices=64, n_he=8, r2d_step=0.05, c2d_step=0.04)
    s = G.Sampler(w, device=0)
    s.run_passes(1, 3)
    s.synchronize()
    s.set_option(OPT_WAIT_NS, 0)
    timed_out = False
    for k in range(8):
        s.run_passes(2, 100 + k)
        try:
            s.synchronize()
        except G.PimcError as e:
            assert e.code == ERR_TIMEOUT, e
            timed_out = True
            break
    assert timed_out, "no rotational wait gave up with a zero limit"
    # the default limit again: passes run, counters advance, estimators are finite
    s.set_option(OPT_WAIT_NS, 2_000_000_000)
    tot0, _ = s.counters()
    s.run_passes(2, 7)
    s.synchronize()
    tot1, _ = s.counters()
    assert tot1[5] - tot0[5] == 2 * w.nslices * w.nrotslices
    est = s.estimators()
    assert np.all(np.isfinite(est))
    s.close()
