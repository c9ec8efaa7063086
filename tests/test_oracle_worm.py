"""The oracle's restatement of the worm algorithm (mc_qworm.cc: open,
close, advance, recede, swap, WorldLine masking of PotEnergy) and of
MCBisectionMoveExchange under the permutations the swaps build, against the
reference run on the same replayed random numbers (tests/golden/c0w.npz).
Same arithmetic in the same order: equal to the last bit."""
import numpy as np

import oracle as O
from _worm import load, replay


def test_worm_sequence_matches_reference():
    w, d, line = load()
    o = O.Oracle(w)
    o.set_state(d["coords0"], d["angles0"], w.pindex)
    o.worm_init(0, line[1], line[2], w.density)

    def bisect(t, time, g, u3):
        st, ds, lv, cons = o.bisection_move(t, time, g, u3, exchange=True)
        assert st == 0
        return cons

    def molec(t, u1, u2):
        st, dv, acc, cons = o.molecular_move(t, u1, u2, exchange=True)
        assert st == 0
        return cons

    cons, states, bcons, mcons = replay(d, lambda s: o.worm_move(s)[1], o.worm_state, bisect, molec)
    np.testing.assert_array_equal(cons, d["w_consumed"])
    np.testing.assert_array_equal(states, d["w_states"])
    np.testing.assert_array_equal(bcons, d["w_bis_cons"])
    np.testing.assert_array_equal(mcons, d["w_mol_cons"])
    c, a, co, p = o.get_state()
    np.testing.assert_array_equal(c, d["coords1"])
    np.testing.assert_array_equal(p, d["pindex1"])
    tot, acc = o.worm_counters()
    np.testing.assert_array_equal(tot[[0, 1, 4, 5, 6]], d["w_total"])
    np.testing.assert_array_equal(acc[[0, 1, 4, 5, 6]], d["w_accep"])
    assert d["w_accep"][4] > 0      # swaps were accepted along the way


def test_exchange_centroid_cycles_match_reference():
    """MCMolecularMoveExchange (mc_piqmc.cc:104-192) with exchange cycles of
    two and three atoms, the reference compiled here against the oracle."""
    import pytest
    if not O.ref_available():
        pytest.skip("the reference is not compiled here")
    w, d, line = load()
    perm = np.arange(w.natoms, dtype=np.int32)
    perm[:6] = [1, 2, 0, 4, 3, 5]
    rng = np.random.default_rng(11)
    ref = O.Reference(w)
    ref.set_state(d["coords1"], d["angles1"], perm)
    o = O.Oracle(w)
    o.set_state(d["coords1"], d["angles1"], perm)
    for k in range(6):
        u1 = rng.uniform(size=18)
        u2 = rng.uniform(size=6) * (0.2 if k % 2 else 1.0)
        ref.replay(u1=u1, u2=u2)
        ref.L.ref_molecular_move_exchange(0)
        pos = ref.replay_pos()
        st, dv, acc, cons = o.molecular_move(0, u1, u2, exchange=True)
        assert st == 0 and tuple(cons) == (pos[0], pos[1])
        c, _, _ = ref.get_state()
        oc, _, _, _ = o.get_state()
        np.testing.assert_array_equal(oc, c)
    tot, accp = ref.counters()
    otot, oacc = o.counters()
    assert tot[0] == otot[0] and accp[0] == oacc[0] and accp[0] > 0
