"""ctypes wrappers for the CPU oracle (oracle/liboracle.so) and for the
reference compiled from its own sources (oracle/_ref/libref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the GB300 library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "moribs-pimc_gb300"))
from pimc_types import BINSC, BINSR, BINST, PimcSystem, PimcTables, dptr, iptr, make_system, make_tables  # noqa: E402

LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_oracle(force=False):
    """Compile oracle/pimc_oracle.c and orc_tables.c into oracle/liboracle.so
    (C11 + OpenMP; libquadmath for the quad-precision type on x86-64).  No
    multiply-add contraction, so that products and sums round as written on
    every host (the reference's x86-64 builds have none)."""
    srcs = [os.path.join(HERE, f) for f in ("pimc_oracle.c", "orc_tables.c")]
    deps = srcs + [os.path.join(HERE, "pimc_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in deps):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"] + srcs + ["-o", LIB, "-lm"]
    if platform.machine() in ("x86_64", "AMD64", "i686"):
        cmd.append("-lquadmath")
    subprocess.check_call(cmd)
    return LIB


LIB_TIMING = os.path.join(HERE, "liboracle_timing.so")


def build_oracle_timing(force=False):
    """The same sources built for speed with the reference's own optimisation
    flags (-Ofast -march=native -fopenmp, makefile.in:3) into
    oracle/liboracle_timing.so: the CPU baseline's build.  Not a parity
    build (fast-math reorders); where the compiler has no -march=native for
    the host (some aarch64 gcc builds), -mcpu=native, then -O3."""
    srcs = [os.path.join(HERE, f) for f in ("pimc_oracle.c", "orc_tables.c")]
    deps = srcs + [os.path.join(HERE, "pimc_oracle.h")]
    if not force and os.path.exists(LIB_TIMING) and all(os.path.getmtime(LIB_TIMING) >= os.path.getmtime(f)
                                                        for f in deps):
        return LIB_TIMING
    tail = srcs + ["-o", LIB_TIMING, "-lm"]
    if platform.machine() in ("x86_64", "AMD64", "i686"):
        tail.append("-lquadmath")
    last = None
    for arch in (["-Ofast", "-march=native"], ["-Ofast", "-mcpu=native"], ["-O3"]):
        cmd = ["gcc", "-std=gnu11", *arch, "-fopenmp", "-fPIC", "-shared"] + tail
        r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
        if r.returncode == 0:
            with open(LIB_TIMING + ".flags", "w") as f:
                f.write(" ".join(arch) + " -fopenmp\n")
            return LIB_TIMING
        last = r.stderr
    raise RuntimeError("timing build of the oracle failed: %s" % last)


def timing_flags():
    try:
        return open(LIB_TIMING + ".flags").read().strip()
    except OSError:
        return None


class Stream(C.Structure):
    _fields_ = [("v", _dp), ("n", C.c_long), ("pos", C.c_long)]


class Replay(C.Structure):
    _fields_ = [("u1", Stream), ("u2", Stream), ("u3", Stream), ("gauss", Stream), ("urot", Stream),
                ("overrun", C.c_int)]


WSTREAMS = ("n1", "n2", "n3", "u1", "u2", "u3", "u4", "u5", "gauss")


class WReplay(C.Structure):
    _fields_ = [(n, Stream) for n in WSTREAMS] + [("overrun", C.c_int)]


def make_wreplay(streams):
    """WReplay over a dict of the worm streams (n1..n3 = nrnd1..3, u1..u5 =
    rnd1..5, gauss); missing streams are empty."""
    keep = []
    rp = WReplay()
    for name in WSTREAMS:
        a = streams.get(name)
        if a is not None:
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            st = getattr(rp, name)
            st.v, st.n, st.pos = dptr(a), len(a), 0
    return rp, keep


def make_replay(u1=None, u2=None, u3=None, gauss=None, urot=None):
    keep = []
    rp = Replay()
    for name, a in (("u1", u1), ("u2", u2), ("u3", u3), ("gauss", gauss), ("urot", urot)):
        st = getattr(rp, name)
        if a is not None:
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            st.v, st.n, st.pos = dptr(a), len(a), 0
    return rp, keep


def _lib(timing=False):
    if timing:
        build_oracle_timing()
    else:
        build_oracle()
    lib = C.CDLL(LIB_TIMING if timing else LIB)
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.POINTER(PimcSystem), C.POINTER(PimcTables), _ip]
    lib.orc_destroy.argtypes = [C.c_void_p]
    for name in ("orc_spot1d",):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_void_p, C.c_double]
    lib.orc_lpot2d.restype = C.c_double
    lib.orc_lpot2d.argtypes = [C.c_void_p, C.c_double, C.c_double]
    lib.orc_srotdens.restype = C.c_double
    lib.orc_srotdens.argtypes = [C.c_void_p, C.c_double, C.c_int]
    lib.orc_vspher.restype = C.c_double
    lib.orc_vspher.argtypes = [C.c_void_p, C.c_double]
    lib.orc_matpre.argtypes = [_dp, _dp]
    lib.orc_deleul.argtypes = [_dp, _dp, _dp]
    lib.orc_rotden.restype = C.c_int
    lib.orc_rotden.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.orc_vcord.restype = C.c_double
    lib.orc_vcord.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.orc_rsrot.argtypes = [_dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, _dp, _dp]
    lib.orc_rsline.argtypes = [C.c_double, C.c_double, C.c_double, _dp, _dp]
    lib.orc_caleng.restype = C.c_double
    lib.orc_caleng.argtypes = [_dp, _dp, _dp, _dp]
    lib.orc_set_state.argtypes = [C.c_void_p, _dp, _dp, _ip]
    lib.orc_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp, _ip]
    for name in ("orc_pot_energy_slice",):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, _dp, C.c_int]
    lib.orc_pot_energy_path.restype = C.c_double
    lib.orc_pot_energy_path.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.orc_pot_rot_energy.restype = C.c_double
    lib.orc_pot_rot_energy.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int]
    lib.orc_pot_rot_e3d.restype = C.c_double
    lib.orc_pot_rot_e3d.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int]
    for name in ("orc_molecular_move", "orc_molecular_move_exchange"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, C.POINTER(Replay), _dp, _ip]
    for name in ("orc_bisection_move", "orc_bisection_move_exchange"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(Replay), _dp, _ip]
    for name in ("orc_rotations_move", "orc_rotations_3d"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, C.POINTER(Replay), _dp, _ip]
    for name in ("orc_rot_lin_step", "orc_rot_3d_step"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _ip]
    lib.orc_get_counters.argtypes = [C.c_void_p, _dp, _dp]
    lib.orc_reset_counters.argtypes = [C.c_void_p]
    for name in ("orc_kin_energy", "orc_pot_energy_est"):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_void_p]
    for name in ("orc_rot_energy", "orc_rot_e3d"):
        getattr(lib, name).restype = C.c_double
        getattr(lib, name).argtypes = [C.c_void_p, _dp, _dp]
    lib.orc_rcf.argtypes = [C.c_void_p, _dp]
    lib.orc_pot_energy_densities.restype = C.c_double
    lib.orc_pot_energy_densities.argtypes = [C.c_void_p, _dp, _dp, _dp]
    lib.orc_exchange_lengths.argtypes = [C.c_void_p, _dp]
    lib.orc_area_estimators.argtypes = [C.c_void_p, _dp]
    lib.orc_area_estim3d.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
    lib.orc_linden.argtypes = [C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
    lib.orc_linden_lmax.argtypes = [C.c_double, C.c_int, C.c_double, _dp]
    lib.orc_rotmat.restype = C.c_double
    lib.orc_rotmat.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
    lib.orc_wigd.restype = C.c_double
    lib.orc_wigd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
    lib.orc_asymrho_energies.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, _dp]
    lib.orc_asymrho_points.argtypes = [C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                       C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
    lib.orc_worm_init.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_double]
    lib.orc_worm_move.argtypes = [C.c_void_p, C.POINTER(WReplay)]
    lib.orc_worm_state.argtypes = [C.c_void_p, _ip]
    lib.orc_worm_set_state.argtypes = [C.c_void_p, _ip]
    lib.orc_worm_counters.argtypes = [C.c_void_p, _dp, _dp]
    lib.orc_worm_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_int, _dp]
    lib.orc_run_steps.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_int, _dp]
    return lib


_LIB = {}


def lib(timing=False):
    if timing not in _LIB:
        _LIB[timing] = _lib(timing)
    return _LIB[timing]


def _v3(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(3))
    return a


class Oracle:
    """One oracle context over a Workload (owns copies of tables and state)."""

    def __init__(self, w, timing=False):
        self.w = w
        self.L = lib(timing)
        self.sys = make_system(w)
        tabs, keep = make_tables(w)
        st = C.c_int(0)
        self.h = self.L.orc_create(C.byref(self.sys), C.byref(tabs), C.byref(st))
        if not self.h:
            raise RuntimeError("orc_create failed: %d" % st.value)
        self.na = w.natoms
        self.P = w.nslices
        if w.coords is not None:
            self.set_state(w.coords, w.angles, w.pindex)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    # state
    def set_state(self, coords, angles=None, pindex=None):
        c = np.ascontiguousarray(coords, dtype=np.float64)
        a = None if angles is None else np.ascontiguousarray(angles, dtype=np.float64)
        p = None if pindex is None else np.ascontiguousarray(pindex, dtype=np.int32)
        self.L.orc_set_state(self.h, dptr(c), dptr(a) if a is not None else None, iptr(p) if p is not None else None)

    def get_state(self):
        nb = self.na * self.P
        c = np.zeros((3, nb)); a = np.zeros((3, nb)); co = np.zeros((3, nb)); p = np.zeros(self.na, np.int32)
        self.L.orc_get_state(self.h, dptr(c), dptr(a), dptr(co), iptr(p))
        return c, a, co, p

    # leaves
    def spot1d(self, r): return self.L.orc_spot1d(self.h, float(r))
    def lpot2d(self, r, c): return self.L.orc_lpot2d(self.h, float(r), float(c))
    def srotdens(self, g, which=0): return self.L.orc_srotdens(self.h, float(g), int(which))
    def vspher(self, r): return self.L.orc_vspher(self.h, float(r))

    def rotden(self, e1, e2):
        e1, e2 = _v3(e1), _v3(e2)
        rel, rho, er, es = np.zeros(3), C.c_double(), C.c_double(), C.c_double()
        st = self.L.orc_rotden(self.h, dptr(e1), dptr(e2), dptr(rel), C.byref(rho), C.byref(er), C.byref(es))
        return st, rel, rho.value, er.value, es.value

    def vcord(self, eul, rcom, rpt):
        e, a, b = _v3(eul), _v3(rcom), _v3(rpt)
        r, t, c = C.c_double(), C.c_double(), C.c_double()
        v = self.L.orc_vcord(self.h, dptr(e), dptr(a), dptr(b), C.byref(r), C.byref(t), C.byref(c))
        return v, r.value, t.value, c.value

    # energies
    def pot_energy_slice(self, atom0, pos, it):
        p = np.ascontiguousarray(pos, dtype=np.float64)
        return self.L.orc_pot_energy_slice(self.h, int(atom0), dptr(p), int(it))

    def pot_energy_path(self, atom0, pos):
        p = np.ascontiguousarray(pos, dtype=np.float64)
        return self.L.orc_pot_energy_path(self.h, int(atom0), dptr(p))

    def pot_rot_energy(self, atom0, cosine, it):
        p = np.ascontiguousarray(cosine, dtype=np.float64)
        return self.L.orc_pot_rot_energy(self.h, int(atom0), dptr(p), int(it))

    def pot_rot_e3d(self, atom0, eul, it):
        e = _v3(eul)
        return self.L.orc_pot_rot_e3d(self.h, int(atom0), dptr(e), int(it))

    # moves
    def molecular_move(self, type_, u1, u2, exchange=False):
        rp, keep = make_replay(u1=u1, u2=u2)
        n = self.w.types[type_]["numb"]
        dv = np.zeros(n); acc = np.zeros(n, np.int32)
        fn = self.L.orc_molecular_move_exchange if exchange else self.L.orc_molecular_move
        st = fn(self.h, type_, C.byref(rp), dptr(dv), iptr(acc))
        return st, dv, acc, (rp.u1.pos, rp.u2.pos)

    def bisection_move(self, type_, time, gauss, u3, exchange=False):
        rp, keep = make_replay(u3=u3, gauss=gauss)
        t = self.w.types[type_]
        ds = np.zeros(t["numb"] * t["levels"]); lv = np.zeros(t["numb"], np.int32)
        fn = self.L.orc_bisection_move_exchange if exchange else self.L.orc_bisection_move
        st = fn(self.h, type_, int(time), C.byref(rp), dptr(ds), iptr(lv))
        return st, ds.reshape(t["numb"], t["levels"]), lv, (rp.gauss.pos, rp.u3.pos)

    # worm algorithm
    def worm_init(self, type_, c, m, density):
        st = self.L.orc_worm_init(self.h, int(type_), float(c), int(m), float(density))
        if st != 0:
            raise RuntimeError("orc_worm_init status %d" % st)

    def worm_move(self, streams):
        rp, keep = make_wreplay(streams)
        st = self.L.orc_worm_move(self.h, C.byref(rp))
        return st, [getattr(rp, n).pos for n in WSTREAMS]

    def worm_run(self, t_begin, t_count, seed, nthreads=1):
        bm = C.c_double()
        st = self.L.orc_worm_run(self.h, int(t_begin), int(t_count), C.c_uint64(seed), int(nthreads), C.byref(bm))
        return st, bm.value

    def worm_state(self):
        st = np.zeros(5, np.int32)
        self.L.orc_worm_state(self.h, iptr(st))
        return st

    def worm_set_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.int32)
        self.L.orc_worm_set_state(self.h, iptr(st))

    def worm_counters(self):
        t, a = np.zeros(7), np.zeros(7)
        self.L.orc_worm_counters(self.h, dptr(t), dptr(a))
        return t, a

    def rotations(self, type_, urot):
        rp, keep = make_replay(urot=urot)
        t = self.w.types[type_]
        n = self.w.nrotslices * t["numb"]
        rd = np.zeros(n); acc = np.zeros(n, np.int32)
        fn = self.L.orc_rotations_move if t["molecule"] == 1 else self.L.orc_rotations_3d
        st = fn(self.h, type_, C.byref(rp), dptr(rd), iptr(acc))
        return st, rd, acc, rp.urot.pos

    def counters(self):
        tot = np.zeros(6); acc = np.zeros(6)
        self.L.orc_get_counters(self.h, dptr(tot), dptr(acc))
        return tot, acc

    # estimators
    def kin_energy(self): return self.L.orc_kin_energy(self.h)
    def pot_energy_est(self): return self.L.orc_pot_energy_est(self.h)

    def rot_energy(self, nonlinear):
        a, b = C.c_double(), C.c_double()
        fn = self.L.orc_rot_e3d if nonlinear else self.L.orc_rot_energy
        s = fn(self.h, C.byref(a), C.byref(b))
        return s, a.value, b.value

    def rcf(self):
        r = np.zeros(self.w.nrotslices)
        self.L.orc_rcf(self.h, dptr(r))
        return r

    def densities(self):
        """(E_pot, gr1d[2,BINSR], gr2d[2,BINSR,BINST], gr3d[2,BINSR*BINST*BINSC]) of this path."""
        g1 = np.zeros((2, BINSR)); g2 = np.zeros((2, BINSR, BINST)); g3 = np.zeros((2, BINSR * BINST * BINSC))
        v = self.L.orc_pot_energy_densities(self.h, dptr(g1), dptr(g2), dptr(g3))
        return v, g1, g2, g3

    def exchange_lengths(self, nboson):
        pl = np.zeros(nboson)
        self.L.orc_exchange_lengths(self.h, dptr(pl))
        return pl

    def area_estimators(self):
        out = np.zeros(6)
        st = self.L.orc_area_estimators(self.h, dptr(out))
        if st != 0:
            raise RuntimeError("orc_area_estimators status %d" % st)
        return out

    def area_estim3d(self, iframe, masses):
        out = np.zeros(18)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        st = self.L.orc_area_estim3d(self.h, int(iframe), dptr(m), dptr(out))
        if st != 0:
            raise RuntimeError("orc_area_estim3d status %d" % st)
        return out

    def run_steps(self, t_begin, t_count, seed, nthreads=1):
        bm = C.c_double()
        st = self.L.orc_run_steps(self.h, int(t_begin), int(t_count), C.c_uint64(seed), int(nthreads), C.byref(bm))
        return st, bm.value


def ref_available():
    return os.path.exists(REFLIB)


class Reference:
    """The reference's own C++ (compiled here from its sources) over one
    workload.  Each instance loads a private copy of libref.so so that the
    reference's global state is per instance."""

    def __init__(self, w, workdir=None):
        sys.path.insert(0, os.path.join(REPO, "moribs-pimc_gb300"))
        from workloads import write_reference_inputs
        self.w = w
        self.tmp = workdir or tempfile.mkdtemp(prefix="pimcref_")
        write_reference_inputs(w, self.tmp)
        libcopy = os.path.join(self.tmp, "libref_copy.so")
        shutil.copy(REFLIB, libcopy)
        L = C.CDLL(libcopy, mode=os.RTLD_LOCAL)
        self.L = L
        L.ref_setup.argtypes = [C.c_char_p]
        L.ref_load_3d.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.ref_load_rho.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int]
        L.ref_load_sph.argtypes = [_dp, C.c_int, C.c_double, C.c_double, C.c_double]
        L.ref_set_state.argtypes = [_dp, _dp, _ip]
        L.ref_get_state.argtypes = [_dp, _dp, _dp]
        L.ref_set_replay.argtypes = [_dp, C.c_long, _dp, C.c_long, _dp, C.c_long, _dp, C.c_long, _dp, C.c_long]
        L.ref_replay_pos.argtypes = [C.POINTER(C.c_long)]
        for n in ("ref_pot_energy_slice",):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_int, _dp, C.c_int]
        L.ref_pot_energy_path.restype = C.c_double
        L.ref_pot_energy_path.argtypes = [C.c_int, _dp]
        L.ref_pot_rot_energy.restype = C.c_double
        L.ref_pot_rot_energy.argtypes = [C.c_int, _dp, C.c_int]
        L.ref_pot_rot_e3d.restype = C.c_double
        L.ref_pot_rot_e3d.argtypes = [C.c_int, _dp, C.c_int]
        L.ref_spot1d.restype = C.c_double
        L.ref_spot1d.argtypes = [C.c_double, C.c_int]
        L.ref_lpot2d.restype = C.c_double
        L.ref_lpot2d.argtypes = [C.c_double, C.c_double, C.c_int]
        L.ref_srotdens.restype = C.c_double
        L.ref_srotdens.argtypes = [C.c_double, C.c_int, C.c_int]
        for n in ("ref_molecular_move", "ref_molecular_move_exchange", "ref_rotations_move", "ref_rotations_3d"):
            getattr(L, n).argtypes = [C.c_int]
        for n in ("ref_bisection_move", "ref_bisection_move_exchange"):
            getattr(L, n).argtypes = [C.c_int, C.c_int]
        for n in ("ref_rot_lin_step", "ref_rot_3d_step"):
            getattr(L, n).argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.ref_counters.argtypes = [_dp, _dp]
        for n in ("ref_kin_energy", "ref_pot_energy_est"):
            getattr(L, n).restype = C.c_double
        for n in ("ref_rot_energy", "ref_rot_e3d"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [_dp, _dp]
        L.ref_set_wreplay.argtypes = sum(([_dp, C.c_long] for _ in range(9)), [])
        L.ref_wreplay_pos.argtypes = [C.POINTER(C.c_long)]
        L.ref_worm_state.argtypes = [_ip]
        L.ref_worm_set_state.argtypes = [_ip]
        L.ref_worm_counters.argtypes = [_dp, _dp]
        L.ref_pindex.argtypes = [_ip, _ip]
        L.ref_mass.restype = C.c_double
        L.ref_mass.argtypes = [C.c_int]
        L.ref_set_pindex.argtypes = [_ip]
        L.ref_densities.restype = C.c_double
        L.ref_densities.argtypes = [_dp, _dp, _dp]
        L.ref_exchange_lengths.argtypes = [_dp]
        L.ref_area_estimators.argtypes = [_dp]
        L.ref_area_estim3d.argtypes = [C.c_int, _dp]
        L.ref_box_size.argtypes = [_dp]
        L.ref_save_densities.argtypes = [C.c_char_p, C.c_double, C.c_int]
        L.ref_save_exchange_length.argtypes = [C.c_char_p, C.c_double, C.c_long]
        L.ref_save_area_estimators.argtypes = [C.c_char_p, C.c_double, C.c_long]
        L.ref_save_area_estim3d.argtypes = [C.c_char_p, C.c_double, C.c_long, C.c_int]
        L.ref_rcf_save.argtypes = [C.c_char_p, C.c_double, C.c_int, _dp]
        L.ref_energy_block.argtypes = [C.c_char_p, C.c_char_p, C.c_long, _dp]
        L.ref_sum_energy.argtypes = [C.c_char_p, C.c_double, _dp]
        L.ref_rel_euler.argtypes = [C.c_char_p, C.c_double, _dp, _dp, _dp]
        L.ref_write_xyz.argtypes = [C.c_char_p]
        L.ref_tau.restype = C.c_double
        L.ref_lambda.restype = C.c_double
        L.ref_lambda.argtypes = [C.c_int]
        cwd = os.getcwd()
        try:
            if L.ref_setup(self.tmp.encode()) != 0:
                raise RuntimeError("ref_setup failed")
        finally:
            os.chdir(cwd)
        tb = w.tables
        self._keep = []
        if "vtable" in tb:
            vt = np.ascontiguousarray(tb["vtable"], dtype=np.float64).ravel()
            self._keep.append(vt)
            L.ref_load_3d(dptr(vt), tb["rgrd"], tb["thgrd"], tb["chgrd"], tb["rvmin"], tb["rvmax"],
                          tb.get("chi_fold_deg", 0))
        if "rhoprp" in tb:
            arrs = [np.ascontiguousarray(tb[k], dtype=np.float64).ravel() for k in ("rhoprp", "erotpr", "erotsq")]
            self._keep += arrs
            L.ref_load_rho(dptr(arrs[0]), dptr(arrs[1]), dptr(arrs[2]), tb["nth"], tb["nph"], tb["nch"])
        if "sph_table" in tb:
            st = np.ascontiguousarray(tb["sph_table"], dtype=np.float64)
            self._keep.append(st)
            L.ref_load_sph(dptr(st), len(st), tb["sph_r0"], tb["sph_rmax"], tb["sph_rstep"])
        self.na = w.natoms
        self.P = w.nslices
        if w.coords is not None:
            self.set_state(w.coords, w.angles, w.pindex)

    def set_state(self, coords, angles, pindex=None):
        c = np.ascontiguousarray(coords, dtype=np.float64)
        a = np.ascontiguousarray(angles, dtype=np.float64)
        p = None if pindex is None else np.ascontiguousarray(pindex, dtype=np.int32)
        self.L.ref_set_state(dptr(c), dptr(a), iptr(p) if p is not None else None)

    def get_state(self):
        nb = self.na * self.P
        c = np.zeros((3, nb)); a = np.zeros((3, nb)); co = np.zeros((3, nb))
        self.L.ref_get_state(dptr(c), dptr(a), dptr(co))
        return c, a, co

    def replay(self, u1=None, u2=None, u3=None, gauss=None, urot=None):
        self._rp = []
        args = []
        for a in (u1, u2, u3, gauss, urot):
            if a is None:
                args += [None, 0]
            else:
                a = np.ascontiguousarray(a, dtype=np.float64)
                self._rp.append(a)
                args += [dptr(a), len(a)]
        self.L.ref_set_replay(*args)

    def replay_pos(self):
        p = (C.c_long * 6)()
        self.L.ref_replay_pos(p)
        return list(p)

    def counters(self):
        tot = np.zeros(6); acc = np.zeros(6)
        self.L.ref_counters(dptr(tot), dptr(acc))
        return tot, acc

    def worm_move(self, streams):
        self._wp = []
        args = []
        for n in WSTREAMS:
            a = streams.get(n)
            if a is None:
                args += [None, 0]
            else:
                a = np.ascontiguousarray(a, dtype=np.float64)
                self._wp.append(a)
                args += [dptr(a), len(a)]
        self.L.ref_set_wreplay(*args)
        self.L.ref_worm_move()
        p = (C.c_long * 10)()
        self.L.ref_wreplay_pos(p)
        return list(p)

    def worm_state(self):
        st = np.zeros(5, np.int32)
        self.L.ref_worm_state(iptr(st))
        return st

    def worm_counters(self):
        t, a = np.zeros(7), np.zeros(7)
        self.L.ref_worm_counters(dptr(t), dptr(a))
        return t, a

    def pindex(self):
        p, r = np.zeros(self.na, np.int32), np.zeros(self.na, np.int32)
        self.L.ref_pindex(iptr(p), iptr(r))
        return p, r

    def set_pindex(self, pindex):
        p = np.ascontiguousarray(pindex, dtype=np.int32)
        self.L.ref_set_pindex(iptr(p))

    def densities(self):
        g1 = np.zeros((2, BINSR)); g2 = np.zeros((2, BINSR, BINST)); g3 = np.zeros((2, BINSR * BINST * BINSC))
        v = self.L.ref_densities(dptr(g1), dptr(g2), dptr(g3))
        return v, g1, g2, g3

    def exchange_lengths(self, nboson):
        pl = np.zeros(nboson)
        self.L.ref_exchange_lengths(dptr(pl))
        return pl

    def area_estimators(self):
        out = np.zeros(6)
        self.L.ref_area_estimators(dptr(out))
        return out

    def area_estim3d(self, iframe):
        out = np.zeros(15)
        self.L.ref_area_estim3d(int(iframe), dptr(out))
        return out

    def box_size(self):
        b = np.zeros(3)
        self.L.ref_box_size(dptr(b))
        return b

    # the reference's block writers on the accumulators last filled above
    def save_densities(self, fname, acount, mode):
        self.L.ref_save_densities(fname.encode(), float(acount), int(mode))

    def save_exchange_length(self, fname, acount, blocknumb):
        self.L.ref_save_exchange_length(fname.encode(), float(acount), int(blocknumb))

    def save_area_estimators(self, fname, acount, blocknumb):
        self.L.ref_save_area_estimators(fname.encode(), float(acount), int(blocknumb))

    def save_area_estim3d(self, fname, acount, blocknumb, iframe):
        self.L.ref_save_area_estim3d(fname.encode(), float(acount), int(blocknumb), int(iframe))

    def energy_block(self, workdir, fname, blocknumb):
        """MCResetBlockAverage, one MCGetAverage (run in workdir), SaveEnergy;
        returns the seven block sums."""
        out = np.zeros(7)
        if self.L.ref_energy_block(str(workdir).encode(), fname.encode(), int(blocknumb), dptr(out)) != 0:
            raise RuntimeError("ref_energy_block failed")
        return out

    def sum_energy(self, workdir, numb):
        """InitTotalAverage, one MCGetAverage, SaveSumEnergy (into
        workdir/<prefix>_sum.eng); returns the seven run totals."""
        out = np.zeros(7)
        if self.L.ref_sum_energy(str(workdir).encode(), float(numb), dptr(out)) != 0:
            raise RuntimeError("ref_sum_energy failed")
        return out

    def rel_euler(self, fname, acount):
        """GetRotE3D's relative-angle histograms of the path and SaveRho1D's
        run-total files (fname_sum.*)."""
        t, p, c = np.zeros(BINST), np.zeros(BINSC), np.zeros(BINSC)
        self.L.ref_rel_euler(fname.encode(), float(acount), dptr(t), dptr(p), dptr(c))
        return t, p, c

    def rcf_save(self, fname, acount, mode):
        """GetRCF on cleared accumulators, then SaveRCF; returns the ten rows written."""
        r = np.zeros((10, self.w.nrotslices))
        self.L.ref_rcf_save(fname.encode(), float(acount), int(mode), dptr(r))
        return r


def linden(temprt, nslice, bconst, npt, iodevn=-1):
    """linear_prop/linden.f: (cost, rho, erot, erotsq) rows, shape (4, npt)."""
    out = np.zeros((4, npt))
    st = lib().orc_linden(float(temprt), int(nslice), float(bconst), int(npt), int(iodevn),
                          dptr(out[0]), dptr(out[1]), dptr(out[2]), dptr(out[3]))
    if st != 0:
        raise RuntimeError("orc_linden status %d" % st)
    return out


def asymrho_points(temprt, nslice, iodevn, abc, maxj, ith, iphi, ichi):
    """nmv_prop/asymrho.f at grid points (degrees): (rho, erot, esq, info[15])."""
    ith, iphi, ichi = (np.ascontiguousarray(a, dtype=np.int32) for a in (ith, iphi, ichi))
    n = len(ith)
    r, e, s, info = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(15)
    st = lib().orc_asymrho_points(float(temprt), int(nslice), int(iodevn), float(abc[0]), float(abc[1]),
                                  float(abc[2]), int(maxj), n, iptr(ith), iptr(iphi), iptr(ichi),
                                  dptr(r), dptr(e), dptr(s), dptr(info))
    if st != 0:
        raise RuntimeError("orc_asymrho_points status %d" % st)
    return r, e, s, info


def asymrho_energies(maxj, abc):
    n = (maxj + 1) * (maxj + 1)
    out = np.zeros(n)
    m = lib().orc_asymrho_energies(int(maxj), float(abc[0]), float(abc[1]), float(abc[2]), dptr(out))
    return out[:m]
