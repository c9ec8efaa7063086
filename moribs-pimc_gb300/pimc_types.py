"""ctypes mirror of include/pimc_types.h and conversion from a Workload."""
from __future__ import annotations

import ctypes as C

import numpy as np

PIMC_MAX_TYPES = 2
# density histogram grids (mc_estim.cc:25-30); mirror of pimc_types.h
BINSR, BINST, BINSC = 300, 50, 100
STATUS = {
    0: "PIMC_OK", 1: "PIMC_ERR_BAD_ARG", 2: "PIMC_ERR_BAD_TABLE", 3: "PIMC_ERR_GRID_RANGE",
    4: "PIMC_ERR_NEG_DENSITY", 5: "PIMC_ERR_TIMEOUT", 6: "PIMC_ERR_CUDA", 7: "PIMC_ERR_NO_DEVICE",
    8: "PIMC_ERR_SIZE", 9: "PIMC_ERR_STATE",
}


class PimcType(C.Structure):
    _fields_ = [("numb", C.c_int), ("molecule", C.c_int), ("stat", C.c_int), ("levels", C.c_int),
                ("mcstep", C.c_double), ("lamb", C.c_double)]


class PimcSystem(C.Structure):
    _fields_ = [("ntypes", C.c_int), ("type", PimcType * PIMC_MAX_TYPES), ("nslices", C.c_int),
                ("nrotslices", C.c_int), ("rotation", C.c_int), ("temperature", C.c_double),
                ("rtstep", C.c_double), ("ispher", C.c_int), ("rot_den_type", C.c_int), ("rot_odevn", C.c_int),
                ("rot_eoff", C.c_double), ("rot_abc", C.c_double * 3), ("rn_ratio", C.c_int),
                ("minimage", C.c_int), ("box", C.c_double * 3)]


_dp = C.POINTER(C.c_double)


class PimcTables(C.Structure):
    _fields_ = [("n1d", C.c_int), ("grid1d", _dp), ("pot1d", _dp),
                ("nr2d", C.c_int), ("nc2d", C.c_int), ("dr2d", C.c_double), ("dc2d", C.c_double),
                ("rgrid2d", _dp), ("cgrid2d", _dp), ("pot2d", _dp),
                ("rgrd", C.c_int), ("thgrd", C.c_int), ("chgrd", C.c_int), ("chi_fold_deg", C.c_int),
                ("rvmin", C.c_double), ("rvmax", C.c_double), ("vtable", _dp),
                ("nrot", C.c_int), ("rotgrid", _dp), ("rotdens", _dp), ("rotderv", _dp), ("rotesqr", _dp),
                ("nth", C.c_int), ("nph", C.c_int), ("nch", C.c_int),
                ("rhoprp", _dp), ("erotpr", _dp), ("erotsq", _dp),
                ("nsph", C.c_int), ("sph_r0", C.c_double), ("sph_rmax", C.c_double), ("sph_rstep", C.c_double),
                ("sph_table", _dp)]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int))


def make_system(w) -> PimcSystem:
    s = PimcSystem()
    s.ntypes = len(w.types)
    for i, t in enumerate(w.types):
        s.type[i].numb = t["numb"]
        s.type[i].molecule = t["molecule"]
        s.type[i].stat = t["stat"]
        s.type[i].levels = t["levels"]
        s.type[i].mcstep = t["mcstep"]
        s.type[i].lamb = t["lamb"]
    s.nslices = w.nslices
    s.nrotslices = w.nrotslices if w.rotation else 0
    s.rotation = 1 if w.rotation else 0
    s.temperature = w.temperature
    s.rtstep = w.rtstep
    s.ispher = w.ispher
    s.rot_den_type = w.rot_den_type
    s.rot_odevn = w.rot_odevn
    s.rot_eoff = w.rot_eoff
    for i in range(3):
        s.rot_abc[i] = w.rot_abc[i]
    s.rn_ratio = w.rn_ratio
    s.minimage = 0
    return s


def make_tables(w):
    """Returns (PimcTables, keepalive list of arrays)."""
    t = PimcTables()
    keep = []
    tb = w.tables

    def arr(name):
        a = np.ascontiguousarray(np.asarray(tb[name], dtype=np.float64).ravel())
        keep.append(a)
        return dptr(a)

    if "grid1d" in tb:
        t.n1d = len(tb["grid1d"])
        t.grid1d, t.pot1d = arr("grid1d"), arr("pot1d")
    if "pot2d" in tb:
        t.nr2d, t.nc2d = len(tb["rgrid2d"]), len(tb["cgrid2d"])
        t.dr2d, t.dc2d = tb["dr2d"], tb["dc2d"]
        t.rgrid2d, t.cgrid2d, t.pot2d = arr("rgrid2d"), arr("cgrid2d"), arr("pot2d")
    if "vtable" in tb:
        t.rgrd, t.thgrd, t.chgrd = tb["rgrd"], tb["thgrd"], tb["chgrd"]
        t.chi_fold_deg = tb.get("chi_fold_deg", 0)
        t.rvmin, t.rvmax = tb["rvmin"], tb["rvmax"]
        t.vtable = arr("vtable")
    if "rotdens" in tb:
        t.nrot = len(tb["rotgrid"])
        t.rotgrid, t.rotdens, t.rotderv, t.rotesqr = arr("rotgrid"), arr("rotdens"), arr("rotderv"), arr("rotesqr")
    if "rhoprp" in tb:
        t.nth, t.nph, t.nch = tb["nth"], tb["nph"], tb["nch"]
        t.rhoprp, t.erotpr, t.erotsq = arr("rhoprp"), arr("erotpr"), arr("erotsq")
    if "sph_table" in tb:
        t.nsph = len(tb["sph_table"])
        t.sph_r0, t.sph_rmax, t.sph_rstep = tb["sph_r0"], tb["sph_rmax"], tb["sph_rstep"]
        t.sph_table = arr("sph_table")
    return t, keep
