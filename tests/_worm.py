"""Replay of the worm fixture (tests/golden/c0w.npz) through any
implementation with worm_move(streams) and bisection_move(type, t, g, u3,
exchange=True)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WSTREAMS = ("n1", "n2", "n3", "u1", "u2", "u3", "u4", "u5", "gauss")


def load():
    import sys
    g = os.path.join(HERE, "golden")
    if g not in sys.path:
        sys.path.insert(0, g)
    import make_golden as M
    return M.make_worm_workload(), dict(np.load(os.path.join(g, "c0w.npz"))), M.WORM_LINE


def split(d, key, nkey):
    n = d[nkey]
    return np.split(d[key], np.cumsum(n)[:-1]) if len(n) else []


def replay(d, worm_move, worm_state, bisect, molec=None):
    """Drive the recorded sequence; returns per-call consumed counts, states,
    the bisection consumption and (with molec) the exchange centroid
    consumption."""
    streams = {n: split(d, "w_" + n, "wn_" + n) for n in WSTREAMS}
    bis_after = {int(k): int(j) for k, j in d["w_bis_after"]}
    nb = len(d["w_bis_t"])
    nbos = 6
    bg = np.split(d["w_bis_gauss"], nb) if nb else []
    bu = np.split(d["w_bis_u3"], nb) if nb else []
    m1 = np.split(d["w_mol_u1"], nb) if nb else []
    m2 = np.split(d["w_mol_u2"], nb) if nb else []
    cons, states, bcons, mcons = [], [], [], []
    for k in range(len(d["w_states"])):
        cons.append(worm_move({n: streams[n][k] for n in WSTREAMS}))
        states.append(worm_state())
        if k in bis_after:
            j = bis_after[k]
            bcons.append(bisect(0, int(d["w_bis_t"][j]), bg[j], bu[j]))
            if molec is not None:
                mcons.append(molec(0, m1[j], m2[j]))
    out = (np.array(cons), np.array(states), np.array(bcons).reshape(-1, 2))
    return out + (np.array(mcons).reshape(-1, 2),) if molec is not None else out
