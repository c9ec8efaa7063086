"""Shared helpers for the tests: fixtures, replay of golden move sequences."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_golden(case):
    import make_golden as M  # tests/golden is on sys.path via load below
    return M


def golden_cases():
    return ["c0s", "c1s", "c3s"]


def golden(case):
    import sys
    if os.path.join(GOLDEN) not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_golden as M
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    w = M.make_workload(case)
    return w, d, M


def split_streams(d):
    out = {}
    for name in ("gauss", "u1", "u2", "u3", "urot"):
        s, n = d["s_" + name], d["n_" + name]
        out[name] = np.split(s, np.cumsum(n)[:-1]) if len(n) else []
    return out


def replay_sequence(d, bisect, molec, rotate):
    """Drive a move implementation through a fixture's sequence.  bisect(typ,
    t, gauss, u3), molec(typ, u1, u2), rotate(typ, urot) perform one
    reference-call each and return the stream positions consumed."""
    st = split_streams(d)
    ib = im = ir = 0
    consumed = []
    for kind, typ, t in d["seq"]:
        if kind == 0:
            consumed.append(bisect(int(typ), int(t), st["gauss"][ib], st["u3"][ib])); ib += 1
        elif kind == 1:
            consumed.append(molec(int(typ), st["u1"][im], st["u2"][im])); im += 1
        else:
            consumed.append(rotate(int(typ), st["urot"][ir])); ir += 1
    return consumed
