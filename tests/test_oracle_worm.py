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

    cons, states, bcons = replay(d, lambda s: o.worm_move(s)[1], o.worm_state, bisect)
    np.testing.assert_array_equal(cons, d["w_consumed"])
    np.testing.assert_array_equal(states, d["w_states"])
    np.testing.assert_array_equal(bcons, d["w_bis_cons"])
    c, a, co, p = o.get_state()
    np.testing.assert_array_equal(c, d["coords1"])
    np.testing.assert_array_equal(p, d["pindex1"])
    tot, acc = o.worm_counters()
    np.testing.assert_array_equal(tot[[0, 1, 4, 5, 6]], d["w_total"])
    np.testing.assert_array_equal(acc[[0, 1, 4, 5, 6]], d["w_accep"])
    assert d["w_accep"][4] > 0      # swaps were accepted along the way
