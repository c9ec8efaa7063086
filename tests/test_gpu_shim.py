"""The reference-name shim's core on the GPU (libpimc_shim.so through ctypes):
the fixture's sequence of reference calls (MCBisectionMove, MCMolecularMove,
MCRotationsMove / MCRotations3D) made through the look-ahead queues from
continuous random streams -- each stream is what the reference drew from it,
call after call -- must reproduce the reference's final path and its
MCTotal / MCAccep counts, and leave exactly the look-ahead values unused.

The fixtures were made by giving the reference one array per call; the
values a call did not reach were never drawn.  Joining the consumed part of
each call's array gives the stream the reference's generator would have
produced for the same decisions."""
import ctypes as C
import os

import numpy as np
import pytest

import pimc_gb300 as G
from _common import golden, split_streams

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(os.path.dirname(HERE), "moribs-pimc_gb300", "libpimc_shim.so")
DRAW = C.CFUNCTYPE(C.c_double, C.c_void_p)


class _Stream:
    def __init__(self, parts):
        self.v = np.concatenate(parts) if parts else np.zeros(0)
        self.i = 0

    def __call__(self, _ctx):
        x = float(self.v[self.i]) if self.i < len(self.v) else 0.5     # past the end: look-ahead only
        self.i += 1
        return x


def _streams(d):
    st = split_streams(d)
    parts = {"gauss": [], "u1": [], "u2": [], "u3": []}
    ib = im = 0
    for (kind, typ, t), cons in zip(d["seq"], d["consumed"]):
        if kind == 0:
            parts["gauss"].append(st["gauss"][ib][:cons[3]]); parts["u3"].append(st["u3"][ib][:cons[2]]); ib += 1
        elif kind == 1:
            parts["u1"].append(st["u1"][im][:cons[0]]); parts["u2"].append(st["u2"][im][:cons[1]]); im += 1
    return {k: _Stream(v) for k, v in parts.items()}, st


@pytest.mark.parametrize("name", ["c0s", "c1s", "c3s", "c4s"])
def test_shim_replays_the_reference_sequence(name):
    w, d, _ = golden(name)
    L = C.CDLL(SHIM)
    L.pimc_shim_create.restype = C.c_void_p
    L.pimc_shim_create.argtypes = [C.c_void_p, DRAW, DRAW, DRAW, DRAW, C.c_void_p]
    L.pimc_shim_destroy.argtypes = [C.c_void_p]
    for f in ("pimc_shim_bisection",):
        getattr(L, f).argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.pimc_shim_molecular.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.pimc_shim_rotations.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_long, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
    L.pimc_shim_pending.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
    s = G.Sampler(w)
    streams, st = _streams(d)
    cb = [DRAW(streams["u1"]), DRAW(streams["u2"]), DRAW(streams["u3"]), DRAW(streams["gauss"])]
    sh = L.pimc_shim_create(s.h, *cb, None)
    assert sh
    total, accep = np.zeros(6), np.zeros(6)
    ir = 0
    for (kind, typ, t), cons in zip(d["seq"], d["consumed"]):
        tt, aa = C.c_double(), C.c_double()
        if kind == 0:
            assert L.pimc_shim_bisection(sh, int(typ), int(t), C.byref(tt), C.byref(aa)) == 0
            k = 3 * int(typ) + 1
        elif kind == 1:
            assert L.pimc_shim_molecular(sh, int(typ), C.byref(tt), C.byref(aa)) == 0
            k = 3 * int(typ) + 0
        else:
            u = np.ascontiguousarray(st["urot"][ir][:cons[4]]); ir += 1
            assert L.pimc_shim_rotations(sh, u.ctypes.data_as(C.POINTER(C.c_double)), len(u), C.byref(tt),
                                         C.byref(aa)) == 0
            k = 3 * int(typ) + 2
        total[k] += tt.value
        accep[k] += aa.value
    c, a, co, _ = s.get_state()
    np.testing.assert_allclose(c, d["coords1"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(a, d["angles1"], rtol=1e-10, atol=1e-12)
    np.testing.assert_array_equal(total[:len(d["total"])], d["total"])
    np.testing.assert_array_equal(accep[:len(d["accep"])], d["accep"])
    # every value the reference drew was used, in order; what is left in the
    # queues is only the look-ahead past the last call
    pend = (C.c_long * 4)()
    L.pimc_shim_pending(sh, pend)
    for name_, q in zip(("u1", "u2", "u3", "gauss"), pend):
        stream = streams[name_]
        assert stream.i - q == len(stream.v), (name_, stream.i, q, len(stream.v))
    L.pimc_shim_destroy(sh)
    s.close()
