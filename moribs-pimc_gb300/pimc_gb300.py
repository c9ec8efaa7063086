"""ctypes binding of libpimc_gb300.so (include/pimc_gb300.h).

This module only marshals arrays; every computation runs in the CUDA
library.  Loading fails loudly when the library has not been built: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from pimc_types import BINSC, BINSR, BINST, PIMC_MAX_TYPES, PimcSystem, PimcTables, STATUS, dptr, iptr, make_system, make_tables

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libpimc_gb300.so")
REPO = os.path.dirname(HERE)
HEADERS = [os.path.join(REPO, "include", "pimc_gb300.h")]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_L = None
OPT_FUSED = 1          # pimc_gb300.h PIMC_OPT_FUSED
OPT_DENSITIES = 2      # pimc_gb300.h PIMC_OPT_DENSITIES


class PimcError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed: %s (%d)" % (what, STATUS.get(code, "?"), code))
        self.code = code


def load(path=LIBPATH):
    """Load the CUDA library; raises if it is missing."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(path):
        raise RuntimeError("libpimc_gb300.so not built at %s: run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    vp = C.c_void_p
    L.pimc_create.argtypes = [C.POINTER(PimcSystem), C.c_int, C.POINTER(vp)]
    L.pimc_destroy.argtypes = [vp]
    L.pimc_load_tables.argtypes = [vp, C.POINTER(PimcTables)]
    L.pimc_set_state.argtypes = [vp, _dp, _dp, _ip]
    L.pimc_get_state.argtypes = [vp, _dp, _dp, _dp, _ip]
    L.pimc_molecular_move.argtypes = [vp, C.c_int, _dp, C.c_long, _dp, C.c_long, _lp, _dp, _ip]
    L.pimc_bisection_move.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp, C.c_long, _dp, C.c_long, _lp, _dp, _ip]
    L.pimc_rotations_move.argtypes = [vp, _dp, C.c_long, _dp, _ip]
    L.pimc_pot_energy.argtypes = [vp, C.c_int, _ip, _ip, _dp, _dp]
    L.pimc_pot_rot_energy.argtypes = [vp, C.c_int, _ip, _ip, _dp, _dp]
    L.pimc_estimators.argtypes = [vp, _dp]
    L.pimc_rcf.argtypes = [vp, _dp]
    L.pimc_molecular_move_exchange.argtypes = [vp, C.c_int, _dp, C.c_long, _dp, C.c_long, _lp]
    L.pimc_worm_init.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_double]
    L.pimc_worm_move.argtypes = [vp, C.POINTER(_dp), C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.pimc_worm_run.argtypes = [vp, C.c_int, C.c_uint64]
    L.pimc_worm_state.argtypes = [vp, _ip]
    L.pimc_worm_set_state.argtypes = [vp, _ip]
    L.pimc_worm_counters.argtypes = [vp, _dp, _dp]
    L.pimc_mlp_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.pimc_mlp_destroy.argtypes = [vp]
    _fp = C.POINTER(C.c_float)
    L.pimc_mlp_set_weights.argtypes = [vp, _fp, _fp, _fp, _fp, _fp, _fp, _fp, C.c_float]
    L.pimc_mlp_forward.argtypes = [vp, C.c_int, _fp, _fp]
    L.pimc_mlp_forward_resident.argtypes = [vp, C.c_int]
    L.pimc_mlp_stream.restype = vp
    L.pimc_mlp_stream.argtypes = [vp]
    L.pimc_mlp_param_count.restype = C.c_int
    L.pimc_mlp_get_params.argtypes = [vp, _fp]
    L.pimc_mlp_gradients.argtypes = [vp, C.c_int, _fp, _fp, _fp, _dp]
    L.pimc_mlp_train.argtypes = [vp, C.c_int, _fp, _fp, C.c_int, C.c_int, C.c_float, C.c_uint64, _dp]
    L.pimc_da_samples.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.pimc_da_sweeps.argtypes = [vp, vp, C.c_int, C.c_uint64, C.c_float, C.c_int, _dp]
    L.pimc_linden.argtypes = [C.c_int, C.c_int, _dp, _ip, C.c_double, C.c_int, C.c_int, _dp]
    sp, cc = C.POINTER(PimcSystem), C.c_char_p
    L.pimc_save_densities_1d.argtypes = [sp, cc, C.c_double, _dp, _dp]
    L.pimc_save_gra_sum.argtypes = [sp, cc, C.c_double, _dp]
    L.pimc_save_rel_euler.argtypes = [sp, cc, C.c_double, _dp, _dp, _dp]
    L.pimc_rel_euler_read.argtypes = [vp, _dp, _dp, _dp]
    for n in ("pimc_save_densities_2d", "pimc_save_densities_3d", "pimc_save_rho_1d", "pimc_save_rho_theta_chi"):
        getattr(L, n).argtypes = [sp, cc, C.c_double, C.c_int, _dp]
    L.pimc_save_exchange_length.argtypes = [sp, cc, C.c_double, C.c_long, C.c_int, _dp, _ip, C.c_int]
    L.pimc_save_area_estimators.argtypes = [sp, cc, C.c_double, C.c_long, C.c_int, _dp, C.c_double]
    L.pimc_save_area_estim3d.argtypes = [sp, cc, C.c_double, C.c_long, C.c_int, C.c_int, _dp, _dp, C.c_double]
    L.pimc_save_rcf.argtypes = [sp, cc, C.c_double, C.c_int, _dp]
    L.pimc_energy_accumulate.argtypes = [sp, _dp, _dp]
    L.pimc_save_energy.argtypes = [sp, cc, C.c_double, C.c_long, _dp]
    L.pimc_blocking_se.argtypes = [_dp, C.c_long, _dp]
    L.pimc_fp64_peak.argtypes = [C.c_int, _dp]
    L.pimc_fp64_probe.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp]
    L.pimc_save_sum_energy.argtypes = [sp, cc, C.c_double, C.c_double, _dp, C.c_int]
    L.pimc_asymrho.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int,
                               _dp, _dp, _dp, _dp]
    L.pimc_densities_accumulate.argtypes = [vp]
    L.pimc_densities_read.argtypes = [vp, _dp, _dp, _dp]
    L.pimc_densities_reset.argtypes = [vp]
    L.pimc_exchange_lengths.argtypes = [vp, _dp]
    L.pimc_area_estimators.argtypes = [vp, _dp]
    L.pimc_area_estim3d.argtypes = [vp, C.c_int, _dp, _dp]
    L.pimc_run_passes.argtypes = [vp, C.c_int, C.c_uint64]
    L.pimc_counters.argtypes = [vp, _dp, _dp]
    L.pimc_profile_pass.argtypes = [vp, C.c_uint64, _dp, C.POINTER(C.c_longlong)]
    L.pimc_reset_counters.argtypes = [vp]
    L.pimc_synchronize.argtypes = [vp]
    L.pimc_set_precision.argtypes = [vp, C.c_int]
    L.pimc_set_option.argtypes = [vp, C.c_int, C.c_longlong]
    L.pimc_bead_moves_per_pass.restype = C.c_double
    L.pimc_bead_moves_per_pass.argtypes = [vp]
    L.pimc_launch_count.restype = C.c_longlong
    L.pimc_launch_count.argtypes = [vp]
    L.pimc_stream.restype = vp
    L.pimc_stream.argtypes = [vp]
    L.pimc_status_string.restype = C.c_char_p
    L.pimc_status_string.argtypes = [C.c_int]
    L.pimc_save_checkpoint.argtypes = [vp, C.c_char_p]
    L.pimc_load_checkpoint.argtypes = [vp, C.c_char_p]
    L.pimc_write_xyz.argtypes = [vp, C.c_char_p, C.c_void_p]
    L.pimc_read_xyz.argtypes = [vp, C.c_char_p]
    # replica batches
    L.pimc_batch_create.argtypes = [C.c_int, C.POINTER(PimcSystem), C.c_int, C.POINTER(vp)]
    L.pimc_batch_destroy.argtypes = [vp]
    L.pimc_batch_load_tables.argtypes = [vp, C.POINTER(PimcTables)]
    L.pimc_batch_set_state.argtypes = [vp, C.c_int, _dp, _dp, _ip]
    L.pimc_batch_get_state.argtypes = [vp, C.c_int, _dp, _dp, _dp, _ip]
    L.pimc_batch_set_precision.argtypes = [vp, C.c_int]
    L.pimc_batch_set_shape.argtypes = [vp, C.c_int, C.c_int]
    L.pimc_batch_autotune.argtypes = [vp, C.c_uint64, _ip, _dp]
    L.pimc_batch_run_passes.argtypes = [vp, C.c_int, C.c_uint64]
    L.pimc_batch_estimators.argtypes = [vp, _dp]
    L.pimc_batch_counters.argtypes = [vp, _dp, _dp]
    L.pimc_batch_synchronize.argtypes = [vp]
    L.pimc_batch_bead_moves_per_pass.restype = C.c_double
    L.pimc_batch_bead_moves_per_pass.argtypes = [vp]
    L.pimc_batch_replica_seed.restype = C.c_uint64
    L.pimc_batch_replica_seed.argtypes = [C.c_uint64, C.c_int]
    L.pimc_batch_stream.restype = vp
    L.pimc_batch_stream.argtypes = [vp]
    L.pimc_batch_set_rotation_mode.argtypes = [vp, C.c_int]
    L.pimc_batch_da_sweeps.argtypes = [vp, vp, C.c_int, C.c_uint64, C.c_float, C.c_int, _dp]
    L.pimc_batch_da_passes.argtypes = [vp, vp, C.c_int, C.c_uint64, C.c_float, C.c_int, _dp]
    _L = L
    return L


def declared_symbols():
    """Names of the functions declared in include/pimc_gb300.h."""
    import re
    names = []
    for h in HEADERS:
        txt = open(h).read()
        names += re.findall(r"^\s*(?:pimc_status|double|long long|void\s*\*|const char\s*\*)\s*(pimc_\w+)\s*\(", txt, re.M)
    return names


def _chk(code, what):
    if code != 0:
        raise PimcError(code, what)


class Sampler:
    """One pimc_handle: a system, its tables and its path on one GPU."""

    def __init__(self, w, device=0, mixed=False):
        self.L = load()
        self.w = w
        self.na = w.natoms
        self.P = w.nslices
        self.sys = make_system(w)
        h = C.c_void_p()
        _chk(self.L.pimc_create(C.byref(self.sys), device, C.byref(h)), "pimc_create")
        self.h = h
        tabs, keep = make_tables(w)
        _chk(self.L.pimc_load_tables(self.h, C.byref(tabs)), "pimc_load_tables")
        if mixed:
            _chk(self.L.pimc_set_precision(self.h, 1), "pimc_set_precision")
        if w.coords is not None:
            self.set_state(w.coords, w.angles, w.pindex)

    def close(self):
        if getattr(self, "h", None):
            self.L.pimc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # path
    def set_state(self, coords=None, angles=None, pindex=None):
        c = None if coords is None else np.ascontiguousarray(coords, dtype=np.float64)
        a = None if angles is None else np.ascontiguousarray(angles, dtype=np.float64)
        p = None if pindex is None else np.ascontiguousarray(pindex, dtype=np.int32)
        _chk(self.L.pimc_set_state(self.h, dptr(c) if c is not None else None, dptr(a) if a is not None else None,
                                   iptr(p) if p is not None else None), "pimc_set_state")

    def get_state(self):
        nb = self.na * self.P
        c = np.zeros((3, nb)); a = np.zeros((3, nb)); co = np.zeros((3, nb)); p = np.zeros(self.na, np.int32)
        _chk(self.L.pimc_get_state(self.h, dptr(c), dptr(a), dptr(co), iptr(p)), "pimc_get_state")
        return c, a, co, p

    # replay moves
    def bisection_move(self, type_, time, gauss, u3, exchange=False):
        g = np.ascontiguousarray(gauss, dtype=np.float64)
        u = np.ascontiguousarray(u3, dtype=np.float64)
        t = self.w.types[type_]
        ds = np.zeros(t["numb"] * t["levels"]); lv = np.zeros(t["numb"], np.int32)
        cons = (C.c_long * 2)()
        st = self.L.pimc_bisection_move(self.h, type_, int(time), int(exchange), dptr(g), len(g), dptr(u), len(u),
                                        cons, dptr(ds), iptr(lv))
        return st, ds.reshape(t["numb"], t["levels"]), lv, (cons[0], cons[1])

    def molecular_move(self, type_, u1, u2):
        a = np.ascontiguousarray(u1, dtype=np.float64)
        b = np.ascontiguousarray(u2, dtype=np.float64)
        n = self.w.types[type_]["numb"]
        dv = np.zeros(n); acc = np.zeros(n, np.int32)
        cons = (C.c_long * 2)()
        st = self.L.pimc_molecular_move(self.h, type_, dptr(a), len(a), dptr(b), len(b), cons, dptr(dv), iptr(acc))
        return st, dv, acc, (cons[0], cons[1])

    def rotations(self, urot):
        u = np.ascontiguousarray(urot, dtype=np.float64)
        rt = [t for t in self.w.types if t["molecule"] != 0][0]
        n = self.w.nrotslices * rt["numb"]
        rd = np.zeros(n); acc = np.zeros(n, np.int32)
        st = self.L.pimc_rotations_move(self.h, dptr(u), len(u), dptr(rd), iptr(acc))
        return st, rd, acc

    # energies
    def pot_energy(self, atom0, it, xyz):
        a = np.ascontiguousarray(atom0, dtype=np.int32)
        t = np.ascontiguousarray(it, dtype=np.int32)
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        out = np.zeros(len(a))
        _chk(self.L.pimc_pot_energy(self.h, len(a), iptr(a), iptr(t), dptr(x), dptr(out)), "pimc_pot_energy")
        return out

    def pot_rot_energy(self, rotor, it, v3):
        a = np.ascontiguousarray(rotor, dtype=np.int32)
        t = np.ascontiguousarray(it, dtype=np.int32)
        x = np.ascontiguousarray(v3, dtype=np.float64).reshape(-1)
        out = np.zeros(len(a))
        _chk(self.L.pimc_pot_rot_energy(self.h, len(a), iptr(a), iptr(t), dptr(x), dptr(out)), "pimc_pot_rot_energy")
        return out

    def estimators(self):
        out = np.zeros(5)
        _chk(self.L.pimc_estimators(self.h, dptr(out)), "pimc_estimators")
        return out

    def rcf(self):
        out = np.zeros(self.w.nrotslices)
        _chk(self.L.pimc_rcf(self.h, dptr(out)), "pimc_rcf")
        return out

    def molecular_move_exchange(self, type_, u1, u2):
        """MCMolecularMoveExchange with replayed rnd1()/rnd2(); returns the draws consumed."""
        a = np.ascontiguousarray(u1, dtype=np.float64)
        b = np.ascontiguousarray(u2, dtype=np.float64)
        cons = (C.c_long * 2)()
        _chk(self.L.pimc_molecular_move_exchange(self.h, int(type_), dptr(a), len(a), dptr(b), len(b), cons),
             "pimc_molecular_move_exchange")
        return (cons[0], cons[1])

    # delayed acceptance with the surrogate (water dimer)
    def da_samples(self):
        f = np.zeros((self.P, 6), dtype=np.float32)
        e = np.zeros(self.P, dtype=np.float32)
        _chk(self.L.pimc_da_samples(self.h, f.ctypes.data_as(C.POINTER(C.c_float)),
                                    e.ctypes.data_as(C.POINTER(C.c_float))), "pimc_da_samples")
        return f, e

    def da_sweeps(self, nsweeps, seed, mlp=None, escale=1.0):
        st = np.zeros(4)
        _chk(self.L.pimc_da_sweeps(self.h, mlp.h if mlp is not None else None, int(nsweeps), C.c_uint64(seed),
                                   C.c_float(escale), 1 if mlp is not None else 0, dptr(st)), "pimc_da_sweeps")
        return st

    # worm algorithm (mc_qworm.cc)
    WSTREAMS = ("n1", "n2", "n3", "u1", "u2", "u3", "u4", "u5", "gauss")

    def worm_init(self, type_, c, m, density):
        _chk(self.L.pimc_worm_init(self.h, int(type_), float(c), int(m), float(density)), "pimc_worm_init")

    def worm_move(self, streams):
        """One MCWormMove with the replay streams of WSTREAMS; returns the draws consumed per stream."""
        arrs = [np.ascontiguousarray(streams.get(n, np.zeros(0)), dtype=np.float64) for n in self.WSTREAMS]
        ptrs = (_dp * 9)(*[dptr(a) if len(a) else _dp() for a in arrs])
        lens = (C.c_long * 9)(*[len(a) for a in arrs])
        used = (C.c_long * 9)()
        _chk(self.L.pimc_worm_move(self.h, ptrs, lens, used), "pimc_worm_move")
        return list(used)

    def worm_run(self, npasses, seed):
        _chk(self.L.pimc_worm_run(self.h, int(npasses), C.c_uint64(seed)), "pimc_worm_run")

    def worm_state(self):
        st = np.zeros(5, np.int32)
        _chk(self.L.pimc_worm_state(self.h, iptr(st)), "pimc_worm_state")
        return st

    def worm_set_state(self, st):
        a = np.ascontiguousarray(st, dtype=np.int32)
        _chk(self.L.pimc_worm_set_state(self.h, iptr(a)), "pimc_worm_set_state")

    def worm_counters(self):
        t, a = np.zeros(7), np.zeros(7)
        _chk(self.L.pimc_worm_counters(self.h, dptr(t), dptr(a)), "pimc_worm_counters")
        return t, a

    def densities_accumulate(self):
        _chk(self.L.pimc_densities_accumulate(self.h), "pimc_densities_accumulate")

    def densities_read(self):
        """(gr1d[2,BINSR], gr2d[2,BINSR,BINST], gr3d[2,BINSR*BINST*BINSC]) accumulated counts."""
        g1 = np.zeros((PIMC_MAX_TYPES, BINSR))
        g2 = np.zeros((PIMC_MAX_TYPES, BINSR, BINST))
        g3 = np.zeros((PIMC_MAX_TYPES, BINSR * BINST * BINSC))
        _chk(self.L.pimc_densities_read(self.h, dptr(g1), dptr(g2), dptr(g3)), "pimc_densities_read")
        return g1, g2, g3

    def rel_euler_read(self):
        """GetRotE3D's relative-Euler-angle histograms (theta, phi, chi)."""
        t, p, c = np.zeros(BINST), np.zeros(BINSC), np.zeros(BINSC)
        _chk(self.L.pimc_rel_euler_read(self.h, dptr(t), dptr(p), dptr(c)), "pimc_rel_euler_read")
        return t, p, c

    def densities_reset(self):
        _chk(self.L.pimc_densities_reset(self.h), "pimc_densities_reset")

    def exchange_lengths(self, ploops=None):
        nb = [t["numb"] for t in self.w.types if t["stat"] == 1][-1]
        out = np.zeros(nb) if ploops is None else ploops
        _chk(self.L.pimc_exchange_lengths(self.h, dptr(out)), "pimc_exchange_lengths")
        return out

    def area_estimators(self):
        out = np.zeros(6)
        _chk(self.L.pimc_area_estimators(self.h, dptr(out)), "pimc_area_estimators")
        return out

    def area_estim3d(self, iframe, masses):
        m = np.ascontiguousarray(masses, dtype=np.float64)
        out = np.zeros(18)
        _chk(self.L.pimc_area_estim3d(self.h, int(iframe), dptr(m), dptr(out)), "pimc_area_estim3d")
        return out

    # production
    def run_passes(self, n, seed):
        _chk(self.L.pimc_run_passes(self.h, int(n), C.c_uint64(seed)), "pimc_run_passes")

    def profile_pass(self, seed):
        ms = np.zeros(3)
        n = (C.c_longlong * 3)()
        _chk(self.L.pimc_profile_pass(self.h, C.c_uint64(seed), dptr(ms), n), "pimc_profile_pass")
        return ms, np.array(list(n))

    def save_checkpoint(self, path):
        _chk(self.L.pimc_save_checkpoint(self.h, str(path).encode()), "pimc_save_checkpoint")

    def load_checkpoint(self, path):
        _chk(self.L.pimc_load_checkpoint(self.h, str(path).encode()), "pimc_load_checkpoint")

    def write_xyz(self, path, type_names=None):
        arr = None
        if type_names:
            arr = (C.c_char_p * len(type_names))(*[n.encode() for n in type_names])
        _chk(self.L.pimc_write_xyz(self.h, str(path).encode(), C.cast(arr, C.c_void_p) if arr else None),
             "pimc_write_xyz")

    def read_xyz(self, path):
        _chk(self.L.pimc_read_xyz(self.h, str(path).encode()), "pimc_read_xyz")

    def set_option(self, option, value):
        _chk(self.L.pimc_set_option(self.h, int(option), int(value)), "pimc_set_option")

    def synchronize(self):
        _chk(self.L.pimc_synchronize(self.h), "pimc_synchronize")

    def counters(self):
        tot = np.zeros(6); acc = np.zeros(6)
        _chk(self.L.pimc_counters(self.h, dptr(tot), dptr(acc)), "pimc_counters")
        return tot, acc

    def reset_counters(self):
        _chk(self.L.pimc_reset_counters(self.h), "pimc_reset_counters")

    def bead_moves_per_pass(self):
        return self.L.pimc_bead_moves_per_pass(self.h)

    def launch_count(self):
        return self.L.pimc_launch_count(self.h)

    def stream(self):
        return self.L.pimc_stream(self.h)


class Batch:
    """A pimc_batch: independent replicas of one species family sampled in
    one persistent launch (include/pimc_gb300.h, replica batches)."""

    def __init__(self, workloads, device=0, mixed=False):
        self.L = load()
        self.ws = list(workloads)
        n = len(self.ws)
        systems = (PimcSystem * n)(*[make_system(w) for w in self.ws])
        h = C.c_void_p()
        _chk(self.L.pimc_batch_create(n, systems, device, C.byref(h)), "pimc_batch_create")
        self.h = h
        tabs = (PimcTables * n)()
        keep = []
        for i, w in enumerate(self.ws):
            t, k = make_tables(w)
            tabs[i] = t
            keep.append(k)
        _chk(self.L.pimc_batch_load_tables(self.h, tabs), "pimc_batch_load_tables")
        if mixed:
            _chk(self.L.pimc_batch_set_precision(self.h, 1), "pimc_batch_set_precision")
        for i, w in enumerate(self.ws):
            self.set_state(i, w.coords, w.angles, w.pindex)

    def close(self):
        if getattr(self, "h", None):
            self.L.pimc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, i, coords, angles, pindex=None):
        c = np.ascontiguousarray(coords, dtype=np.float64)
        a = np.ascontiguousarray(angles, dtype=np.float64)
        p = None if pindex is None else np.ascontiguousarray(pindex, dtype=np.int32)
        _chk(self.L.pimc_batch_set_state(self.h, int(i), dptr(c), dptr(a), iptr(p) if p is not None else None),
             "pimc_batch_set_state")

    def get_state(self, i):
        w = self.ws[i]
        n = w.natoms * w.nslices
        c = np.zeros((3, n)); a = np.zeros((3, n)); co = np.zeros((3, n)); p = np.zeros(w.natoms, np.int32)
        _chk(self.L.pimc_batch_get_state(self.h, int(i), dptr(c), dptr(a), dptr(co), iptr(p)), "pimc_batch_get_state")
        return c, a, co, p

    def set_shape(self, warps, min_blocks=2):
        _chk(self.L.pimc_batch_set_shape(self.h, int(warps), int(min_blocks)), "pimc_batch_set_shape")

    def set_rotation_mode(self, mode):
        _chk(self.L.pimc_batch_set_rotation_mode(self.h, int(mode)), "pimc_batch_set_rotation_mode")

    def autotune(self, seed):
        """(warps, min_blocks) of the fastest shape and the six times (ms per pass)."""
        wo = np.zeros(2, np.int32); ms = np.zeros(6)
        _chk(self.L.pimc_batch_autotune(self.h, C.c_uint64(seed), iptr(wo), dptr(ms)), "pimc_batch_autotune")
        return (int(wo[0]), int(wo[1])), ms

    def run_passes(self, n, seed):
        _chk(self.L.pimc_batch_run_passes(self.h, int(n), C.c_uint64(seed)), "pimc_batch_run_passes")

    def estimators(self):
        out = np.zeros((len(self.ws), 4))
        _chk(self.L.pimc_batch_estimators(self.h, dptr(out)), "pimc_batch_estimators")
        return out

    def counters(self):
        tot = np.zeros(6); acc = np.zeros(6)
        _chk(self.L.pimc_batch_counters(self.h, dptr(tot), dptr(acc)), "pimc_batch_counters")
        return tot, acc

    def synchronize(self):
        _chk(self.L.pimc_batch_synchronize(self.h), "pimc_batch_synchronize")

    def bead_moves_per_pass(self):
        return self.L.pimc_batch_bead_moves_per_pass(self.h)

    def stream(self):
        return self.L.pimc_batch_stream(self.h)

    def da_sweeps(self, nsweeps, seed, mlp=None, escale=1.0):
        st = np.zeros(4)
        _chk(self.L.pimc_batch_da_sweeps(self.h, mlp.h if mlp is not None else None, int(nsweeps), C.c_uint64(seed),
                                         C.c_float(escale), 1 if mlp is not None else 0, dptr(st)), "pimc_batch_da_sweeps")
        return st

    def da_passes(self, npasses, seed, mlp=None, escale=1.0):
        st = np.zeros(4)
        _chk(self.L.pimc_batch_da_passes(self.h, mlp.h if mlp is not None else None, int(npasses), C.c_uint64(seed),
                                         C.c_float(escale), 1 if mlp is not None else 0, dptr(st)), "pimc_batch_da_passes")
        return st

    @staticmethod
    def replica_seed(seed, r):
        return int(load().pimc_batch_replica_seed(C.c_uint64(seed), int(r)))


def blocking_se(x):
    """pimc_blocking_se: dict of mean, sd, naive SE, blocked SE, the
    statistical inefficiency g (2 tau_int, in samples), the block size chosen,
    whether the level test passed, and the number of values used."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(8)
    _chk(load().pimc_blocking_se(dptr(x), len(x), dptr(out)), "pimc_blocking_se")
    return {"mean": out[0], "sd": out[1], "se_naive": out[2], "se": out[3], "g": out[4],
            "block": int(out[5]), "converged": bool(out[6]), "n": int(out[7])}


def fp64_peak(device=0):
    """pimc_fp64_peak: the measured FP64 FMA rate in GFLOP/s."""
    g = np.zeros(1)
    _chk(load().pimc_fp64_peak(int(device), dptr(g)), "pimc_fp64_peak")
    return float(g[0])


def fp64_probe(warps, lanes, iters=20000, device=0):
    """pimc_fp64_probe: device milliseconds of one CTA per SM of `warps`
    warps with `lanes` active lanes, 8 FMA chains of `iters` steps each."""
    ms = C.c_double()
    _chk(load().pimc_fp64_probe(int(device), int(warps), int(lanes), int(iters), C.byref(ms)), "pimc_fp64_probe")
    return ms.value


def linden(temperatures, nslices, bconst, npt, iodevn=-1, device=0):
    """pimc_linden: exact linear-rotor propagator tables (linear_prop/linden.f)
    for each (temperature, nslice) pair; shape (n, 4, npt) with rows cos gamma,
    rho, erot, erotsq."""
    L = load()
    T = np.ascontiguousarray(np.atleast_1d(temperatures), dtype=np.float64)
    ns = np.ascontiguousarray(np.broadcast_to(np.atleast_1d(nslices), T.shape), dtype=np.int32)
    out = np.zeros((len(T), 4, int(npt)))
    _chk(L.pimc_linden(int(device), len(T), dptr(T), iptr(ns), float(bconst), int(npt), int(iodevn), dptr(out)),
         "pimc_linden")
    return out


def asymrho(temperature, nslice, iodevn, ith0, ith1, abc, maxj, device=0):
    """pimc_asymrho: exact asymmetric-top propagator (nmv_prop/asymrho.f) on
    the 1-degree grid for theta ith0..ith1: (rho, erot, esq) each of shape
    (ith1-ith0+1, 361, 361), and info[15]."""
    L = load()
    n = int(ith1) - int(ith0) + 1
    rho, erot, esq = (np.zeros((n, 361, 361)) for _ in range(3))
    info = np.zeros(15)
    a = np.ascontiguousarray(abc, dtype=np.float64)
    _chk(L.pimc_asymrho(int(device), float(temperature), int(nslice), int(iodevn), int(ith0), int(ith1), dptr(a),
                        int(maxj), dptr(rho), dptr(erot), dptr(esq), dptr(info)), "pimc_asymrho")
    return rho, erot, esq, info


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """The tcgen05 surrogate MLP 6 -> 256 -> 256 -> 256 -> 1 (include/pimc_gb300.h)."""

    def __init__(self, device=0):
        self.L = load()
        self.h = C.c_void_p()
        _chk(self.L.pimc_mlp_create(int(device), C.byref(self.h)), "pimc_mlp_create")

    def set_weights(self, w1, b1, w2, b2, w3, b3, w4, b4):
        arrs = [_f32(a) for a in (w1, b1, w2, b2, w3, b3, w4)]
        assert arrs[0].shape == (6, 256) and arrs[2].shape == (256, 256) and arrs[4].shape == (256, 256)
        _chk(self.L.pimc_mlp_set_weights(self.h, *[_fptr(a) for a in arrs], C.c_float(float(b4))),
             "pimc_mlp_set_weights")

    def forward(self, x):
        x = _f32(x).reshape(-1, 6)
        y = np.zeros(len(x), dtype=np.float32)
        _chk(self.L.pimc_mlp_forward(self.h, len(x), _fptr(x), _fptr(y)), "pimc_mlp_forward")
        return y

    def forward_resident(self, n):
        _chk(self.L.pimc_mlp_forward_resident(self.h, int(n)), "pimc_mlp_forward_resident")

    def stream(self):
        return self.L.pimc_mlp_stream(self.h)

    def params(self):
        p = np.zeros(self.L.pimc_mlp_param_count(), dtype=np.float32)
        _chk(self.L.pimc_mlp_get_params(self.h, _fptr(p)), "pimc_mlp_get_params")
        return p

    def gradients(self, x, e):
        x = _f32(x).reshape(-1, 6)
        e = _f32(e)
        g = np.zeros(self.L.pimc_mlp_param_count(), dtype=np.float32)
        loss = C.c_double()
        _chk(self.L.pimc_mlp_gradients(self.h, len(x), _fptr(x), _fptr(e), _fptr(g), C.byref(loss)),
             "pimc_mlp_gradients")
        return g, loss.value

    def train(self, x, e, epochs, batch, lr, seed=0):
        x = _f32(x).reshape(-1, 6)
        e = _f32(e)
        losses = np.zeros(epochs)
        _chk(self.L.pimc_mlp_train(self.h, len(x), _fptr(x), _fptr(e), int(epochs), int(batch), C.c_float(lr),
                                   C.c_uint64(seed), dptr(losses)), "pimc_mlp_train")
        return losses

    def close(self):
        if self.h:
            self.L.pimc_mlp_destroy(self.h)
            self.h = C.c_void_p()


# ---- block files of the estimators (host only)

def _sysbox(w, box):
    s = make_system(w)
    for i in range(3):
        s.box[i] = float(box[i])
    return s


def _arr(a, n=None):
    if a is None:
        return None
    return dptr(np.ascontiguousarray(a, dtype=np.float64))


def save_densities(w, box, fname, acount, mode, gr1d, gr2d, gr3d):
    """The density files of one block (mode 0) or of the run (mode 1):
    SaveDensities1D (block) or SaveGraSum (run), SaveDensities2D,
    SaveDensities3D, SaveRho1D and SaveRhoThetaChi (block) as the reference's
    block and run ends call them
    (mc_main.cc:715-734, 445-460).  gr?d as Sampler.densities_read returns
    them; box = the reference's BoxSize."""
    L = load()
    s = _sysbox(w, box)
    keep = [np.ascontiguousarray(g, dtype=np.float64) for g in (gr1d, gr2d, gr3d)]
    p1, p2, p3 = (dptr(k) for k in keep)
    fn = fname.encode()
    if mode == 0:
        _chk(L.pimc_save_densities_1d(C.byref(s), fn, float(acount), p1, p2), "pimc_save_densities_1d")
    else:
        _chk(L.pimc_save_gra_sum(C.byref(s), fn, float(acount), p1), "pimc_save_gra_sum")
    _chk(L.pimc_save_densities_2d(C.byref(s), fn, float(acount), int(mode), p2), "pimc_save_densities_2d")
    _chk(L.pimc_save_densities_3d(C.byref(s), fn, float(acount), int(mode), p3), "pimc_save_densities_3d")
    _chk(L.pimc_save_rho_1d(C.byref(s), fn, float(acount), int(mode), p3), "pimc_save_rho_1d")
    if mode == 0:
        _chk(L.pimc_save_rho_theta_chi(C.byref(s), fn, float(acount), int(mode), p3), "pimc_save_rho_theta_chi")


def save_exchange_length(w, fname, acount, blocknumb, bstype, ploops, pindex, print_xyz_prl=0):
    L = load()
    s = make_system(w)
    pl = np.ascontiguousarray(ploops, dtype=np.float64)
    pi = np.ascontiguousarray(pindex, dtype=np.int32)
    _chk(L.pimc_save_exchange_length(C.byref(s), fname.encode(), float(acount), int(blocknumb), int(bstype),
                                     dptr(pl), iptr(pi), int(print_xyz_prl)), "pimc_save_exchange_length")


def save_area_estimators(w, fname, acount, blocknumb, bstype, sums, mass):
    L = load()
    s = make_system(w)
    sm = np.ascontiguousarray(sums, dtype=np.float64)
    _chk(L.pimc_save_area_estimators(C.byref(s), fname.encode(), float(acount), int(blocknumb), int(bstype),
                                     dptr(sm), float(mass)), "pimc_save_area_estimators")


def save_area_estim3d(w, fname, acount, blocknumb, iframe, bstype, areas, inert, mass):
    L = load()
    s = make_system(w)
    a = np.ascontiguousarray(areas, dtype=np.float64)
    i = np.ascontiguousarray(inert, dtype=np.float64)
    _chk(L.pimc_save_area_estim3d(C.byref(s), fname.encode(), float(acount), int(blocknumb), int(iframe),
                                  int(bstype), dptr(a), dptr(i), float(mass)), "pimc_save_area_estim3d")


def save_rcf(w, fname, acount, mode, rcf):
    L = load()
    s = make_system(w)
    r = np.ascontiguousarray(rcf, dtype=np.float64)
    _chk(L.pimc_save_rcf(C.byref(s), fname.encode(), float(acount), int(mode), dptr(r)), "pimc_save_rcf")


def energy_accumulate(w, est, sums=None):
    """MCGetAverage's energy terms of one sample added to sums[7] (returned)."""
    L = load()
    s = make_system(w)
    e = np.ascontiguousarray(est, dtype=np.float64)
    out = np.zeros(7) if sums is None else np.ascontiguousarray(sums, dtype=np.float64)
    _chk(L.pimc_energy_accumulate(C.byref(s), dptr(e), dptr(out)), "pimc_energy_accumulate")
    return out


def save_energy(w, fname, acount, blocknumb, sums):
    L = load()
    s = make_system(w)
    sm = np.ascontiguousarray(sums, dtype=np.float64)
    _chk(L.pimc_save_energy(C.byref(s), fname.encode(), float(acount), int(blocknumb), dptr(sm)),
         "pimc_save_energy")


def save_sum_energy(w, fname, acount, numb, sums, append=False):
    L = load()
    s = make_system(w)
    sm = np.ascontiguousarray(sums, dtype=np.float64)
    _chk(L.pimc_save_sum_energy(C.byref(s), fname.encode(), float(acount), float(numb), dptr(sm), int(bool(append))),
         "pimc_save_sum_energy")




def save_rel_euler(w, fname, acount, the, phi, chi):
    L = load()
    s = make_system(w)
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (the, phi, chi)]
    _chk(L.pimc_save_rel_euler(C.byref(s), fname.encode(), float(acount), dptr(a[0]), dptr(a[1]), dptr(a[2])),
         "pimc_save_rel_euler")

