"""CPU-side checks of the C-ABI library: it loads, exports every symbol that
include/pimc_gb300.h declares, and rejects work without a GPU."""
import ctypes as C
import os

import pytest

import pimc_gb300 as G

pytestmark = pytest.mark.skipif(not os.path.exists(G.LIBPATH), reason="library not built (__graft_entry__.build())")


def test_exports_every_declared_symbol():
    L = G.load()
    names = G.declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n


def test_status_strings():
    L = G.load()
    for code in range(10):
        assert L.pimc_status_string(code)


def test_create_validates_before_touching_a_device():
    import workloads as W
    L = G.load()
    w = W.config0(seed=1, nslices=16, nrotslices=4, n_he=2)
    s = G.make_system(w)
    s.type[0].levels = 5          # 2^5 >= P: rejected like MCInit (mc_setup.cc:397-398)
    h = C.c_void_p()
    assert L.pimc_create(C.byref(s), 0, C.byref(h)) == 1
    s = G.make_system(w)
    s.nrotslices = 5              # P not divisible by Q (mc_setup.cc:382-389)
    assert L.pimc_create(C.byref(s), 0, C.byref(h)) == 1
