"""The allocation-free PotEnergy query (pimc_pot_energy_noalloc) against the
allocating one (pimc_pot_energy), through the C ABI, on two calls in a row.

Some callers cannot let the library allocate device memory once they are set
up (they own the device memory through their own pool or run under a fixed
budget); pimc_pot_energy_noalloc serves them from a fixed array inside the
library.  This file is collected last so that a run stopping at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import pimc_gb300 as G
from _common import golden

pytestmark = pytest.mark.gpu
MAX_QUERIES = 4096


def _bind(L):
    f = L.pimc_pot_energy_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                  C.POINTER(C.c_double)]
    f.restype = C.c_int
    g = L.pimc_pot_energy
    g.argtypes = f.argtypes
    g.restype = C.c_int
    return f, g


def _queries(w, rng, n):
    P = w.nslices
    a0 = rng.integers(0, w.natoms, n).astype(np.int32)
    it = rng.integers(0, P, n).astype(np.int32)
    xyz = np.ascontiguousarray(
        np.array([w.coords[:, a * P + t] + rng.normal(0.0, 0.1, 3) for a, t in zip(a0, it)]), dtype=np.float64)
    return a0, it, xyz


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    w, d, _ = golden("c1s")
    s = G.Sampler(w)
    noalloc, alloc = _bind(s.L)
    rng = np.random.default_rng(31)
    for n in (300, 777):                       # two calls in a row, different sizes and contents
        a0, it, xyz = _queries(w, rng, n)
        ref = np.zeros(n)
        got = np.full(n, np.nan)
        assert alloc(s.h, n, G.iptr(a0), G.iptr(it), G.dptr(xyz), G.dptr(ref)) == 0
        assert noalloc(s.h, n, G.iptr(a0), G.iptr(it), G.dptr(xyz), G.dptr(got)) == 0
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)
    s.close()


def test_noalloc_rejects_more_queries_than_the_array_holds():
    w, d, _ = golden("c0s")
    s = G.Sampler(w)
    noalloc, _ = _bind(s.L)
    n = MAX_QUERIES + 1
    a0 = np.zeros(n, np.int32)
    it = np.zeros(n, np.int32)
    xyz = np.zeros(3 * n)
    out = np.zeros(n)
    assert noalloc(s.h, n, G.iptr(a0), G.iptr(it), G.dptr(xyz), G.dptr(out)) == 8   # PIMC_ERR_SIZE
    s.close()


def test_noalloc_matches_the_reference_fixture():
    """The same entry point on the reference's own PotEnergy(atom, pos, it)
    values of the c1s fixture (initial and displaced beads), 1e-10."""
    w, d, _ = golden("c1s")
    s = G.Sampler(w)
    s.set_state(d["coords0"], d["angles0"], w.pindex)
    noalloc, _ = _bind(s.L)
    P = w.nslices
    a0, it, xyz, ref = [], [], [], []
    for a in range(w.natoms):
        for j, t in enumerate(d["slices"]):
            for k, arr in enumerate((d["coords0"], d["pos"])):
                a0.append(a); it.append(int(t)); xyz.append(arr[:, a * P + t]); ref.append(d["e_slice"][a, j, k])
    a0 = np.array(a0, np.int32); it = np.array(it, np.int32)
    xyz = np.ascontiguousarray(np.array(xyz), dtype=np.float64)
    ref = np.array(ref)
    got = np.full(len(ref), np.nan)
    assert noalloc(s.h, len(ref), G.iptr(a0), G.iptr(it), G.dptr(xyz), G.dptr(got)) == 0
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12)
    s.close()
