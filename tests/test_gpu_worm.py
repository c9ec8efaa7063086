"""The worm algorithm on the GPU (pimc_worm_move: open, close, advance,
recede, swap with WorldLine masking) and the exchange bisection under the
permutations it builds, against the reference's own run on the same replayed
random numbers (tests/golden/c0w.npz) and against the oracle.

The potential sums run in another order than the reference's, so paths agree
to 1e-10 relative; every decision, every stream position and the
permutation agree exactly."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
from _worm import WSTREAMS, load, replay, split

pytestmark = pytest.mark.gpu


def _gpu(w, d, line):
    s = G.Sampler(w)
    s.set_state(d["coords0"], d["angles0"], w.pindex)
    s.worm_init(0, line[1], line[2], w.density)
    return s


def test_worm_sequence_matches_reference():
    w, d, line = load()
    s = _gpu(w, d, line)

    def bisect(t, time, g, u3):
        rs, ds, lv, cons = s.bisection_move(t, time, g, u3, exchange=True)
        assert rs == 0
        return cons

    cons, states, bcons, mcons = replay(d, s.worm_move, s.worm_state, bisect, s.molecular_move_exchange)
    np.testing.assert_array_equal(cons, d["w_consumed"])
    np.testing.assert_array_equal(states, d["w_states"])
    np.testing.assert_array_equal(bcons, d["w_bis_cons"])
    np.testing.assert_array_equal(mcons, d["w_mol_cons"])
    c, a, co, p = s.get_state()
    np.testing.assert_allclose(c, d["coords1"], rtol=1e-10, atol=1e-10)
    np.testing.assert_array_equal(p, d["pindex1"])
    tot, acc = s.worm_counters()
    np.testing.assert_array_equal(tot[[0, 1, 4, 5, 6]], d["w_total"])
    np.testing.assert_array_equal(acc[[0, 1, 4, 5, 6]], d["w_accep"])
    s.close()


def test_exchange_bisection_across_the_ring_matches_oracle():
    """Windows that cross the end of the ring join the bead rows through the
    permutation (here the one the recorded worm run ends with, or a cycle of
    all bosons); the GPU and the oracle evaluate each moved bead's own energy
    (the reference's midpoint term reads another atom's row there,
    mc_piqmc.cc:373-376)."""
    w, d, line = load()
    nbos = w.types[0]["numb"]
    rng = np.random.default_rng(5)
    perms = [np.array(d["pindex1"], dtype=np.int32)]
    cyc = np.arange(w.natoms, dtype=np.int32)
    cyc[:nbos] = np.roll(np.arange(nbos), 1)
    perms.append(cyc)
    tested = 0
    for perm in perms:
        if np.array_equal(perm[:nbos], np.arange(nbos)):
            continue
        s = G.Sampler(w)
        s.set_state(d["coords1"], d["angles1"], perm)
        o = O.Oracle(w)
        o.set_state(d["coords1"], d["angles1"], perm)
        for time in range(w.nslices - 8, w.nslices):          # every window across the ring
            g = rng.normal(0.0, 1.0 / np.sqrt(2.0), 3 * nbos * 8)
            u3 = rng.uniform(size=nbos * 3)
            rs, ds, lv, cons = s.bisection_move(0, time, g, u3, exchange=True)
            ost, ods, olv, ocons = o.bisection_move(0, time, g, u3, exchange=True)
            assert rs == 0 and ost == 0
            np.testing.assert_array_equal(lv, olv)
            assert tuple(cons) == tuple(ocons)
            scale = np.maximum(np.abs(ods), 1.0)
            assert np.all(np.abs(ds - ods) <= 1e-9 * scale)
            c, _, _, _ = s.get_state()
            oc, _, _, _ = o.get_state()
            np.testing.assert_allclose(c, oc, rtol=1e-10, atol=1e-10)
            o.set_state(c)           # keep the two paths identical bit for bit
            tested += 1
        s.close()
    assert tested >= 8


def test_exchange_centroid_cycles_match_oracle():
    """MCMolecularMoveExchange with cycles of two and three atoms: the GPU
    against the oracle (which equals the reference bit for bit, see
    tests/test_oracle_worm.py)."""
    w, d, line = load()
    perm = np.arange(w.natoms, dtype=np.int32)
    perm[:6] = [1, 2, 0, 4, 3, 5]
    rng = np.random.default_rng(11)
    s = G.Sampler(w)
    s.set_state(d["coords1"], d["angles1"], perm)
    o = O.Oracle(w)
    o.set_state(d["coords1"], d["angles1"], perm)
    for k in range(6):
        u1 = rng.uniform(size=18)
        u2 = rng.uniform(size=6) * (0.2 if k % 2 else 1.0)
        cons = s.molecular_move_exchange(0, u1, u2)
        st, dv, acc, ocons = o.molecular_move(0, u1, u2, exchange=True)
        assert st == 0 and tuple(cons) == tuple(ocons)
        c, _, _, _ = s.get_state()
        oc, _, _, _ = o.get_state()
        np.testing.assert_allclose(c, oc, rtol=1e-10, atol=1e-10)
        o.set_state(c)
    tot, acc = s.counters()
    otot, oacc = o.counters()
    assert tot[0] == otot[0] and acc[0] == oacc[0] and acc[0] > 0
    s.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_worm_run_production(mixed):
    """The worm branch of the pass loop with counter-based draws on the
    config-0 family (CO2-like rotor + 6 He-4 bosons, P = 32, Q = 8): the same
    seed gives the same path, permutation and worm on a second handle; the
    worm opens, closes and swaps; the path stays finite and the permutation
    a permutation."""
    w, d, line = load()
    runs = []
    for rep in range(2):
        s = G.Sampler(w, mixed=mixed)
        s.set_state(d["coords0"], d["angles0"], w.pindex)
        s.worm_init(0, line[1], line[2], w.density)
        s.worm_run(6, seed=4242)
        c, a, co, p = s.get_state()
        runs.append((c, a, p, s.worm_state(), s.worm_counters(), s.counters()))
        s.close()
    (c0, a0, p0, st0, wc0, mc0), (c1, a1, p1, st1, wc1, mc1) = runs
    np.testing.assert_array_equal(c0, c1)
    np.testing.assert_array_equal(a0, a1)
    np.testing.assert_array_equal(p0, p1)
    np.testing.assert_array_equal(st0, st1)
    assert np.isfinite(c0).all()
    assert sorted(p0[:6]) == list(range(6))
    tot, acc = wc0
    assert tot[0] > 0 and acc[0] > 0 and tot[1] > 0 and acc[1] > 0     # opened and closed
    assert tot[6] > 0                                                  # swaps tried
    mtot, macc = mc0
    assert mtot[5] > 0 and macc[5] > 0                                 # rotor moved
