"""Synthetic MoRiBS-PIMC systems with the shapes of the benchmark configurations.

No datasets or table files travel with this repository, so every table is
generated here from a published functional form, seeded, and written (when
asked) in the reference's own file formats so that the reference readers
(mc_poten.cc:305-546, mc_input.cc:71-515) accept them unchanged:

* He-He: Aziz HFDHE2 form (Aziz et al., J. Chem. Phys. 70, 4330 (1979)) on a
  uniform 1-30 A grid -- the 1D `.pot` format read by init_pot1D
  (mc_poten.cc:379-438).
* pH2-pH2: Silvera-Goldman form (Silvera & Goldman, J. Chem. Phys. 69, 4209
  (1978)) on 1.5-30 A.
* linear rotor - atom: V(r,cos t) = V0(r) (1 + 0.3 P2 + 0.05 P4), V0 a
  Lennard-Jones form -- the 2D `.pot` format of init_pot2D
  (mc_poten.cc:305-377).
* nonlinear rotor - atom: a Lennard-Jones form whose sigma and epsilon carry
  an l <= 6 real spherical-harmonic expansion (even m, cos(m chi): the C2v
  folding of vcord.f:77-85) with seeded Gaussian coefficients of decreasing
  width, tabulated on (r [bohr], theta [deg], chi [deg]) like vcalc expects.
* linear rotor density: the exact free-rotor propagator sum of
  linear_prop/linden.f:88-122 (exarho), the 4-column `.rot` format.
* asymmetric-top density: the rattle-and-shake propagator of
  rotden.f:257-284 (rho = exp(sumaxs / 4 tau)) tabulated on a
  (theta, phi, chi) grid, with its energy estimator; this stands in for the
  exact asymmetric-top sum of nmv_prop/asymrho.f.

Sizes, temperatures and slice counts follow the benchmark configurations.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# physical constants of mc_const.h:11-18,44-50 and mc_setup.cc:207
HBAR = 1.05457266
AMU = 1.6605402
K_B = 1.380658
WNO2K = 0.6950356
LAMBDA_CONST = 100.0 * (HBAR * HBAR) / (AMU * K_B)   # A^2 K amu
MASS_H1 = 1.0078
MASS_H2 = 2.015650642
MASS_HE4 = 4.0026032497
MASS_C12 = 12.0
MASS_O16 = 15.994915
MASS_S32 = 31.972
BOHR_A = 0.52917721092
HARTREE_K = 315774.65

# masses of MCInitParams (mc_setup.cc:244-319)
MASSES = {
    "He4": MASS_HE4,
    "H2": MASS_H2,
    "CO2": MASS_C12 + 2.0 * MASS_O16,
    "SO2": 2.0 * MASS_O16 + MASS_S32,
    "H2O": 2.0 * MASS_H1 + MASS_O16,
}


def lam(mass: float) -> float:
    """hbar^2/2m in K*A^2 exactly as MCSetUnits computes it (mc_setup.cc:207-215)."""
    return 0.5 * LAMBDA_CONST / mass


# ----------------------------------------------------------------- potentials

def aziz_hfdhe2(r):
    """He-He HFDHE2 potential in K, r in A."""
    eps, rm = 10.8, 2.9673
    A, alpha = 0.5448504e6, 13.353384
    c6, c8, c10, D = 1.3732412, 0.4253785, 0.178100, 1.241314
    x = np.asarray(r, dtype=np.float64) / rm
    F = np.where(x < D, np.exp(-(D / x - 1.0) ** 2), 1.0)
    return eps * (A * np.exp(-alpha * x) - (c6 / x**6 + c8 / x**8 + c10 / x**10) * F)


def silvera_goldman(r):
    """pH2-pH2 Silvera-Goldman potential in K, r in A."""
    a, b, g = 1.713, 1.5671, 0.00993
    c6, c8, c9, c10, rc = 12.14, 215.2, 143.1, 4813.9, 8.321
    x = np.asarray(r, dtype=np.float64) / BOHR_A
    fc = np.where(x <= rc, np.exp(-(rc / x - 1.0) ** 2), 1.0)
    v = np.exp(a - b * x - g * x * x) - (c6 / x**6 + c8 / x**8 - c9 / x**9 + c10 / x**10) * fc
    return v * HARTREE_K


def lj(r, eps, sigma):
    s6 = (sigma / np.asarray(r, dtype=np.float64)) ** 6
    return 4.0 * eps * (s6 * s6 - s6)


def legendre(l, x):
    x = np.asarray(x, dtype=np.float64)
    p0, p1 = np.ones_like(x), x
    if l == 0:
        return p0
    for k in range(1, l):
        p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
    return p1


def assoc_legendre(l, m, x):
    """P_l^m(x) by the standard upward recursion (Condon-Shortley phase omitted)."""
    x = np.asarray(x, dtype=np.float64)
    pmm = np.ones_like(x)
    if m > 0:
        somx2 = np.sqrt(np.maximum(0.0, (1.0 - x) * (1.0 + x)))
        fact = 1.0
        for _ in range(m):
            pmm = pmm * fact * somx2
            fact += 2.0
    if l == m:
        return pmm
    pmmp1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmmp1
    for ll in range(m + 2, l + 1):
        pll = (x * (2 * ll - 1) * pmmp1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pmmp1 = pmmp1, pll
    return pmmp1


def rotor_atom_3d(rgrid_bohr, nth, nch, chi_fold_deg, seed, eps0=40.0, sigma0=3.5, lmax=6):
    """V(r, theta, chi) in K on r [bohr] x theta 0..180 [nth] x chi 0..fold [nch]."""
    rng = np.random.default_rng(seed)
    th = np.radians(np.linspace(0.0, 180.0, nth))
    ch = np.radians(np.linspace(0.0, float(chi_fold_deg), nch))
    T, C = np.meshgrid(th, ch, indexing="ij")
    ct = np.cos(T)
    ssig = np.zeros_like(T)
    seps = np.zeros_like(T)
    for l in range(1, lmax + 1):
        width = 0.06 / l
        for m in range(0, l + 1, 2):
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
            y = norm * assoc_legendre(l, m, ct) * np.cos(m * C)
            ssig += rng.normal(0.0, width) * y
            seps += rng.normal(0.0, 2.5 * width) * y
    ssig = np.clip(ssig, -0.15, 0.15)
    seps = np.clip(seps, -0.5, 0.5)
    r_a = np.asarray(rgrid_bohr, dtype=np.float64) * BOHR_A
    sig = sigma0 * (1.0 + ssig)
    eps = eps0 * (1.0 + seps)
    s6 = (sig[None, :, :] / r_a[:, None, None]) ** 6
    v = 4.0 * eps[None, :, :] * (s6 * s6 - s6)
    return np.ascontiguousarray(np.minimum(v, 2.0e5))


def rotor_atom_2d(rgrid, cgrid, eps=30.0, sigma=3.4):
    """V(r, cos t) = V0(r)(1 + 0.3 P2 + 0.05 P4), V0 Lennard-Jones (K, A)."""
    v0 = lj(np.asarray(rgrid), eps, sigma)
    ang = 1.0 + 0.3 * legendre(2, cgrid) + 0.05 * legendre(4, cgrid)
    return np.ascontiguousarray(v0[:, None] * ang[None, :])


# --------------------------------------------------------- rotational tables

def linden_exarho(cost, tau_cm, bconst, nslice, iodevn=-1, maxl=500, eps=1.0e-16):
    """Exact linear-rotor propagator columns (rho, erot, erotsq) of
    linear_prop/linden.f:26-37 (lmax) and exarho (linden.f:88-122)."""
    lmax = maxl
    for l in range(maxl + 1):
        if math.exp(-tau_cm * bconst * l * (l + 1)) < eps:
            lmax = l
            break
    boltz = 0.69503476
    cost = np.asarray(cost, dtype=np.float64)
    rho = np.zeros_like(cost)
    erot = np.zeros_like(cost)
    erotsq = np.zeros_like(cost)
    p_prev, p_cur = np.ones_like(cost), cost.copy()
    for l in range(0, lmax + 1):
        if l == 0:
            pl = p_prev
        elif l == 1:
            pl = p_cur
        else:
            p_next = ((2.0 * (l - 1) + 1) * cost * p_cur - (l - 1) * p_prev) / l
            p_prev, p_cur = p_cur, p_next
            pl = p_cur
        if (l % 2) == iodevn or iodevn == -1:
            tmp = (2 * l + 1) * pl * math.exp(-tau_cm * bconst * float(l * (l + 1)))
            rho += tmp
            erot += tmp * l * (l + 1) * bconst
            erotsq += tmp * l * (l + 1) * bconst * l * (l + 1) * bconst
    erot = erot / (nslice * boltz)
    erotsq = erotsq / (nslice * boltz) ** 2.0
    return rho / (4.0 * math.pi), erot / (4.0 * math.pi), erotsq / (4.0 * math.pi)


def matpre(phi, theta, chi):
    """ZYZ rotation matrix of rotden.f:136-163, broadcasting over arrays."""
    cp, sp, ct, st, ck, sk = np.cos(phi), np.sin(phi), np.cos(theta), np.sin(theta), np.cos(chi), np.sin(chi)
    return np.array([
        [cp * ct * ck - sp * sk, -cp * ct * sk - sp * ck, cp * st],
        [sp * ct * ck + cp * sk, -sp * ct * sk + cp * ck, sp * st],
        [-st * ck, st * sk, ct],
    ])


def rs_top_density(nth, nph, nch, abc, tau_rot_k, scale=1.0):
    """(rho, erot [cm^-1], erot^2) of the rattle-and-shake asymmetric-top
    propagator (rotden.f:247-284) at relative Euler angles on a grid of
    theta 0..180, phi 0..360, chi 0..360 degrees."""
    tau = tau_rot_k / WNO2K
    bl = 1.0 / np.asarray(abc, dtype=np.float64)
    th = np.radians(np.linspace(0.0, 180.0, nth))
    ph = np.radians(np.linspace(0.0, 360.0, nph))
    ch = np.radians(np.linspace(0.0, 360.0, nch))
    T, Pp, C = np.meshgrid(th, ph, ch, indexing="ij")
    m = matpre(Pp, T, C)
    d = [m[0, 0], m[1, 1], m[2, 2]]
    sumaxs = ((bl[0] - bl[1] - bl[2]) * (1.0 - d[0]) + (bl[1] - bl[2] - bl[0]) * (1.0 - d[1])
              + (bl[2] - bl[0] - bl[1]) * (1.0 - d[2]))
    rho = scale * np.exp(sumaxs / (4.0 * tau))
    erot = sumaxs / (4.0 * tau * tau) + 1.5 / tau + 0.25 * float(np.sum(abc))
    return (np.ascontiguousarray(rho), np.ascontiguousarray(erot), np.ascontiguousarray(erot * erot))


# ------------------------------------------------------------------- systems

@dataclass
class Workload:
    """A complete system: parameters, tables and an initial path."""
    name: str
    types: list                    # list of dicts: name, numb, molecule, stat, levels, mcstep, lambda
    nslices: int
    nrotslices: int
    temperature: float
    rtstep: float = 0.0
    rotation: bool = False
    ispher: int = 0
    rot_den_type: int = 0
    rot_odevn: int = -1
    rot_eoff: float = 0.0
    rot_abc: tuple = (0.0, 0.0, 0.0)
    rn_ratio: int = 1
    tables: dict = field(default_factory=dict)
    coords: np.ndarray | None = None   # [3, natoms*P]
    angles: np.ndarray | None = None   # [3, natoms*P]
    pindex: np.ndarray | None = None
    chi_fold_deg: int = 0
    worm: tuple | None = None          # (type name, c, m) of the WORM input line
    density: float = 0.02               # DENSITY of qmc.input (the worm's normalisation)

    @property
    def natoms(self) -> int:
        return sum(t["numb"] for t in self.types)

    def bead_moves_per_pass(self) -> float:
        """Scheduled bead-moves of one pass of the reference schedule
        (mc_main.cc:348-381): per type N*P*(2^L-1) bisection + N*P centroid,
        plus P*Q rotational slice attempts per rotor."""
        P = self.nslices
        bm = 0.0
        for t in self.types:
            bm += t["numb"] * P * ((1 << t["levels"]) - 1) + t["numb"] * P
            if t["molecule"] != 0 and self.rotation:
                bm += t["numb"] * P * self.nrotslices
        return bm


def _sphere_points(rng, n, radius, min_sep, avoid=((0.0, 0.0, 0.0),), avoid_sep=3.0):
    pts = []
    tries = 0
    while len(pts) < n:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place particles")
        p = rng.uniform(-radius, radius, 3)
        if np.dot(p, p) > radius * radius:
            continue
        if any(np.linalg.norm(p - np.asarray(a)) < avoid_sep for a in avoid):
            continue
        if any(np.linalg.norm(p - q) < min_sep for q in pts):
            continue
        pts.append(p)
    return np.array(pts)


def initial_path(natoms, P, positions, rng, jitter=0.02, nrot_first=None):
    """Replicate positions along imaginary time (MCConfigInit, mc_setup.cc:455-489)
    with a small seeded jitter; orientations theta=0 (cos=1), phi=chi=0."""
    coords = np.zeros((3, natoms * P))
    for a in range(natoms):
        for d in range(3):
            coords[d, a * P:(a + 1) * P] = positions[a, d] + rng.normal(0.0, jitter, P)
    angles = np.zeros((3, natoms * P))
    angles[1, :] = 1.0
    return coords, angles


def _table_1d(fn, r0, r1, n):
    g = np.linspace(r0, r1, n)
    return g, fn(g)


def config0(seed=1234, nslices=512, nrotslices=128, n_he=8, r2d_step=0.01, c2d_step=0.01):
    """1 linear CO2-like rotor (B=0.39 cm^-1) + 8 He-4 at 0.37 K."""
    T = 0.37
    types = [
        dict(name="He4", numb=n_he, molecule=0, stat=1, levels=3, mcstep=0.30, lamb=lam(MASSES["He4"]), fpot="he4"),
        dict(name="CO2", numb=1, molecule=1, stat=0, levels=3, mcstep=0.10, lamb=lam(MASSES["CO2"]), fpot="co2he"),
    ]
    g1, v1 = _table_1d(aziz_hfdhe2, 1.0, 30.0, 512)
    nr = int(round(18.0 / r2d_step)) + 1
    nc = int(round(2.0 / c2d_step)) + 1
    rg = np.round(np.arange(nr) * r2d_step + 2.0, 10)
    cg = np.round(np.arange(nc) * c2d_step - 1.0, 10)
    v2 = rotor_atom_2d(rg, cg)
    tau_cm = 1.4387752224 / (T * nrotslices)
    cost = np.array([(ic - 1) * (2.0 / 1499.0) - 1.0 for ic in range(1, 1501)])
    rho, er, esq = linden_exarho(cost, tau_cm, 0.39, nrotslices)
    tables = dict(grid1d=g1, pot1d=v1, rgrid2d=rg, cgrid2d=cg, pot2d=v2, dr2d=r2d_step, dc2d=c2d_step,
                  rotgrid=cost, rotdens=rho, rotderv=er, rotesqr=esq)
    rng = np.random.default_rng(seed)
    pos = _sphere_points(rng, n_he, 10.0, 2.6, avoid=((0, 0, 0),), avoid_sep=3.3)
    pos = np.vstack([pos, np.zeros((1, 3))])
    coords, angles = initial_path(n_he + 1, nslices, pos, rng)
    return Workload("config0-CO2-8He", types, nslices, nrotslices, T, rtstep=0.3, rotation=True,
                    tables=tables, coords=coords, angles=angles, pindex=np.arange(n_he + 1, dtype=np.int32))


def linden_exarho_many(cost, taus_cm, bconst, nslices, maxl=500, eps=1.0e-16):
    """linden_exarho for many propagator times at once (one row per tau):
    every row sums the same Legendre series up to the largest tau's cut-off
    (the extra terms are below eps of the first)."""
    taus = np.asarray(taus_cm, dtype=np.float64)
    tmin = float(taus.min())
    lmax = maxl
    for l in range(maxl + 1):
        if math.exp(-tmin * bconst * l * (l + 1)) < eps:
            lmax = l
            break
    boltz = 0.69503476
    cost = np.asarray(cost, dtype=np.float64)
    rho = np.zeros((len(taus), len(cost)))
    erot = np.zeros_like(rho)
    erotsq = np.zeros_like(rho)
    p_prev, p_cur = np.ones_like(cost), cost.copy()
    for l in range(0, lmax + 1):
        if l == 0:
            pl = p_prev
        elif l == 1:
            pl = p_cur
        else:
            p_next = ((2.0 * (l - 1) + 1) * cost * p_cur - (l - 1) * p_prev) / l
            p_prev, p_cur = p_cur, p_next
            pl = p_cur
        w = (2 * l + 1) * np.exp(-taus * bconst * float(l * (l + 1)))
        tmp = np.outer(w, pl)
        rho += tmp
        erot += tmp * l * (l + 1) * bconst
        erotsq += tmp * (l * (l + 1) * bconst) ** 2
    ns = np.asarray(nslices, dtype=np.float64)[:, None]
    erot = erot / (ns * boltz)
    erotsq = erotsq / (ns * boltz) ** 2
    return rho / (4.0 * math.pi), erot / (4.0 * math.pi), erotsq / (4.0 * math.pi)


def config2(n=4096, seed=2024, p_choices=(64, 128, 256, 512), n_he=(1, 64), t_range=(0.3, 2.0),
            r2d_step=0.01, c2d_step=0.01):
    """n independent replicas of the config-0 family: 1 linear CO2-like rotor
    (B = 0.39 cm^-1) + N He-4, N uniform in n_he, P from p_choices, Q = P/4,
    T uniform in t_range, each seeded.  The He-He and rotor-He tables are
    shared; each replica has its own linear-rotor propagator at
    tau = 1/(T Q)."""
    rng = np.random.default_rng(seed)
    g1, v1 = _table_1d(aziz_hfdhe2, 1.0, 30.0, 512)
    nr = int(round(18.0 / r2d_step)) + 1
    nc = int(round(2.0 / c2d_step)) + 1
    rg = np.round(np.arange(nr) * r2d_step + 2.0, 10)
    cg = np.round(np.arange(nc) * c2d_step - 1.0, 10)
    v2 = rotor_atom_2d(rg, cg)
    ns = rng.integers(n_he[0], n_he[1] + 1, size=n)
    ps = rng.choice(np.asarray(p_choices), size=n)
    ts = rng.uniform(t_range[0], t_range[1], size=n)
    qs = ps // 4
    taus = 1.4387752224 / (ts * qs)
    cost = np.array([(ic - 1) * (2.0 / 1499.0) - 1.0 for ic in range(1, 1501)])
    rho, er, esq = linden_exarho_many(cost, taus, 0.39, qs)
    out = []
    for r in range(n):
        n_r, P, Q, T = int(ns[r]), int(ps[r]), int(qs[r]), float(ts[r])
        types = [
            dict(name="He4", numb=n_r, molecule=0, stat=1, levels=3, mcstep=0.30, lamb=lam(MASSES["He4"]), fpot="he4"),
            dict(name="CO2", numb=1, molecule=1, stat=0, levels=3, mcstep=0.10, lamb=lam(MASSES["CO2"]),
                 fpot="co2he"),
        ]
        tables = dict(grid1d=g1, pot1d=v1, rgrid2d=rg, cgrid2d=cg, pot2d=v2, dr2d=r2d_step, dc2d=c2d_step,
                      rotgrid=cost, rotdens=rho[r], rotderv=er[r], rotesqr=esq[r])
        rr = np.random.default_rng([seed, r])
        radius = 10.0 * (max(n_r, 8) / 8.0) ** (1.0 / 3.0)
        pos = _sphere_points(rr, n_r, radius, 2.6, avoid=((0, 0, 0),), avoid_sep=3.3)
        pos = np.vstack([pos, np.zeros((1, 3))])
        coords, angles = initial_path(n_r + 1, P, pos, rr)
        out.append(Workload("config2-replica-%d" % r, types, P, Q, T, rtstep=0.3, rotation=True,
                            tables=tables, coords=coords, angles=angles, pindex=np.arange(n_r + 1, dtype=np.int32)))
    return out


def config1(seed=4321, nslices=1024, nrotslices=256, n_h2=64, grid3d=(200, 60, 60), griddens=(61, 121, 121),
            ispher=0):
    """1 asymmetric-top SO2-like rotor (A,B,C = 2.03, 0.344, 0.293 cm^-1) + 64 pH2 at 0.37 K.
    ispher 1: the rotor-pH2 pair terms of the translational moves use the
    spherical table of vspher.f (ISPHER, mc_piqmc.cc:1913-1922), here a
    Lennard-Jones form on 3-26 bohr; the rotational moves keep vcord."""
    T = 0.37
    types = [
        dict(name="H2", numb=n_h2, molecule=0, stat=1, levels=3, mcstep=0.20, lamb=lam(MASSES["H2"]), fpot="h2h2"),
        dict(name="SO2", numb=1, molecule=2, stat=0, levels=3, mcstep=0.15, lamb=lam(MASSES["SO2"]), fpot="so2h2"),
    ]
    g1, v1 = _table_1d(silvera_goldman, 1.5, 30.0, 1024)
    nr, nth, nch = grid3d
    rvmin, rvmax = 3.0, 30.0
    rgrid = np.linspace(rvmin, rvmax, nr)
    vt = rotor_atom_3d(rgrid, nth, nch, 90, seed + 7)
    abc = (2.03, 0.344, 0.293)
    tau_rot = 1.0 / (T * nrotslices)
    rho, er, esq = rs_top_density(*griddens, abc, tau_rot)
    tables = dict(grid1d=g1, pot1d=v1, rgrd=nr, thgrd=nth, chgrd=nch, rvmin=rvmin, rvmax=rvmax,
                  vtable=vt, chi_fold_deg=90, nth=griddens[0], nph=griddens[1], nch=griddens[2],
                  rhoprp=rho, erotpr=er, erotsq=esq)
    rng = np.random.default_rng(seed)
    radius = 4.2 * (n_h2 / 8.0) ** (1.0 / 3.0) + 3.0
    pos = _sphere_points(rng, n_h2, radius, 2.9, avoid=((0, 0, 0),), avoid_sep=3.6)
    pos = np.vstack([pos, np.zeros((1, 3))])
    coords, angles = initial_path(n_h2 + 1, nslices, pos, rng)
    if ispher:
        rb = 3.0 + 0.046 * np.arange(501)
        tables.update(sph_table=np.ascontiguousarray(np.minimum(lj(rb * BOHR_A, 40.0, 3.5), 2.0e5)), sph_r0=3.0,
                      sph_rmax=26.0, sph_rstep=0.046)
    return Workload("config1-SO2-64pH2", types, nslices, nrotslices, T, rtstep=0.1, rotation=True,
                    rot_abc=abc, tables=tables, coords=coords, angles=angles, ispher=ispher,
                    pindex=np.arange(n_h2 + 1, dtype=np.int32), chi_fold_deg=90)


def config3(seed=77, nslices=4096, nrotslices=2048, griddens=(61, 121, 121), sep=3.0, rot_den_type=0, levels=5,
            tables=None):
    """2 rigid water-like asymmetric tops (A,B,C = 27.9, 14.5, 9.3 cm^-1) at 0.74 K, caleng potential.
    rot_den_type 1: the analytic rattle-and-shake propagator (ROTDENSI 1) in
    the moves; the table is still loaded for the E^2 estimator."""
    T = 0.74
    types = [dict(name="H2O", numb=2, molecule=2, stat=0, levels=levels, mcstep=0.05, lamb=lam(MASSES["H2O"]),
                  fpot="none")]
    abc = (27.9, 14.5, 9.3)
    tau_rot = 1.0 / (T * nrotslices)
    if tables is None:       # else the density tables of another dimer of the same T and Q
        rho, er, esq = rs_top_density(*griddens, abc, tau_rot)
        tables = dict(nth=griddens[0], nph=griddens[1], nch=griddens[2], rhoprp=rho, erotpr=er, erotsq=esq)
    rng = np.random.default_rng(seed)
    pos = np.array([[0.0, 0.0, 0.0], [sep, 0.0, 0.0]])
    coords, angles = initial_path(2, nslices, pos, rng, jitter=0.01)
    # a hydrogen-bonded start: donor rotated so one H points at the acceptor
    angles[0, :] = 0.0
    angles[1, :] = math.cos(math.radians(127.0))
    return Workload("config3-H2O-dimer", types, nslices, nrotslices, T, rtstep=0.05, rotation=True,
                    rot_abc=abc, tables=tables, coords=coords, angles=angles, rot_den_type=rot_den_type,
                    pindex=np.arange(2, dtype=np.int32))


WATER_ABC = (27.9, 14.5, 9.3)


def water_chain_tables(seed=4040, grid3d=(200, 60, 60)):
    """Potentials shared by every replica of the water-chain family: the
    pH2-pH2 Silvera-Goldman spline (1.5-30 A, 1024 points) and a water-pH2
    V(r, theta, chi) from the same l <= 6 generator as the SO2-pH2 table, with
    its own seed (the water-pH2 surface is not specified; this stands in)."""
    g1, v1 = _table_1d(silvera_goldman, 1.5, 30.0, 1024)
    nr, nth, nch = grid3d
    rvmin, rvmax = 3.0, 30.0
    rgrid = np.linspace(rvmin, rvmax, nr)
    vt = rotor_atom_3d(rgrid, nth, nch, 90, seed + 7, eps0=45.0, sigma0=3.2)
    return dict(grid1d=g1, pot1d=v1, rgrd=nr, thgrd=nth, chgrd=nch, rvmin=rvmin, rvmax=rvmax, vtable=vt,
                chi_fold_deg=90)


def water_chain(nrot, nh2, nslices, nrotslices, T, seed, tables, spacing=3.0, rtstep=0.3, griddens=None,
                name="water-chain"):
    """nrot rigid water-like tops (A, B, C = 27.9, 14.5, 9.3 cm^-1, caleng
    between them) on a linear chain along x with `spacing` A between
    neighbours, solvated by nh2 para-H2 bosons (possibly none), at T.  The
    rotational propagator is the analytic rattle-and-shake one (ROTDENSI 1,
    rotden.f:218-286) at the replica's own tau, so no density table is
    needed; griddens=(nth, nph, nch) also tabulates it (the reference's
    GetRotE3D reads the tabulated E^2 estimator even then)."""
    types = [
        dict(name="H2", numb=nh2, molecule=0, stat=1, levels=3, mcstep=0.20, lamb=lam(MASSES["H2"]), fpot="h2h2"),
        dict(name="H2O", numb=nrot, molecule=2, stat=0, levels=3, mcstep=0.05, lamb=lam(MASSES["H2O"]),
             fpot="h2oh2"),
    ]
    tb = dict(tables)
    if griddens is not None:
        rho, er, esq = rs_top_density(*griddens, WATER_ABC, 1.0 / (T * nrotslices))
        tb.update(nth=griddens[0], nph=griddens[1], nch=griddens[2], rhoprp=rho, erotpr=er, erotsq=esq)
    rng = np.random.default_rng(seed)
    xs = (np.arange(nrot) - 0.5 * (nrot - 1)) * spacing
    wpos = np.stack([xs, np.zeros(nrot), np.zeros(nrot)], axis=1)
    radius = 0.5 * spacing * (nrot - 1) + 4.0 + 2.2 * (max(nh2, 1) / 8.0) ** (1.0 / 3.0)
    hpos = _sphere_points(rng, nh2, radius, 2.9, avoid=[tuple(p) for p in wpos], avoid_sep=3.4) if nh2 else \
        np.zeros((0, 3))
    pos = np.vstack([hpos, wpos])
    coords, angles = initial_path(nh2 + nrot, nslices, pos, rng, jitter=0.01)
    # alternate orientations along the chain: even waters along z, odd ones
    # tilted so that one H points at the next oxygen
    for k in range(nrot):
        a = (nh2 + k) * nslices
        angles[1, a:a + nslices] = 1.0 if k % 2 == 0 else math.cos(math.radians(127.0))
    return Workload(name, types, nslices, nrotslices, T, rtstep=rtstep, rotation=True, rot_den_type=1,
                    rot_abc=WATER_ABC, tables=tb, coords=coords, angles=angles,
                    pindex=np.arange(nh2 + nrot, dtype=np.int32), chi_fold_deg=90)


def water_chain_case(seed, nrot, nh2, nslices, nrotslices, T, grid3d=(30, 37, 19), griddens=None):
    """One system of the water-chain family with its own (small) tables."""
    return water_chain(nrot, nh2, nslices, nrotslices, T, seed, water_chain_tables(seed, grid3d), griddens=griddens,
                       name="water-chain-%dw-%dh2" % (nrot, nh2))


def config4(n=512, seed=4040, p_choices=(512, 1024, 2048), n_rot=(1, 8), n_h2=(0, 32), t_range=(0.5, 2.0),
            grid3d=(200, 60, 60)):
    """n independent replicas of the water-chain family: per replica the
    number of waters (n_rot), of pH2 (n_h2), the temperature (t_range) and
    the translational slices (p_choices, rotational slices P/4: 512-2048 and
    128-512) drawn from the seed; shared potential tables."""
    rng = np.random.default_rng(seed)
    tables = water_chain_tables(seed, grid3d)
    nr = rng.integers(n_rot[0], n_rot[1] + 1, size=n)
    nh = rng.integers(n_h2[0], n_h2[1] + 1, size=n)
    ps = rng.choice(np.asarray(p_choices), size=n)
    ts = rng.uniform(t_range[0], t_range[1], size=n)
    return [water_chain(int(nr[r]), int(nh[r]), int(ps[r]), int(ps[r]) // 4, float(ts[r]), [seed, r], tables,
                        rtstep=0.1, name="config4-replica-%d" % r) for r in range(n)]


# ------------------------------------------------ reference file formats

def _fmt_temperature(T):
    """stringstream << double with default precision 6 (mc_poten.cc:445-446)."""
    return "%g" % T


def write_reference_inputs(w: Workload, workdir: str, passes=1, blocks=1):
    """qmc.input plus the 1D/2D potential and .rot files the reference reads."""
    os.makedirs(workdir, exist_ok=True)
    lines = ["MASTERDIR ./", "OUTPUTDIR ./", "FILENAMEPREFIX ref", "DIMENSION 3",
             "DENSITY %r" % w.density, "TEMPERATURE %r" % w.temperature]
    for t in w.types:
        kw = "ATOM" if t["molecule"] == 0 else ("MOLECULE" if t["molecule"] == 1 else "NONLINEAR")
        stat = "BOSE" if t["stat"] == 1 else "BOLTZMANN"
        numb = -t["numb"] if (w.ispher and t["molecule"] != 0) else t["numb"]
        lines.append("%s %s %d %s %r %d %s PRIMITIVE" % (kw, t["name"], numb, stat, t["mcstep"], t["levels"], t["fpot"]))
    if w.rotation:
        rt = [t for t in w.types if t["molecule"] != 0][0]
        lines.append("ROTATION %s %r %d" % (rt["name"], w.rtstep, w.nrotslices))
        lines.append("ROTDENSI %d %d %r %r %r %r %d" % (w.rot_den_type, w.rot_odevn, w.rot_eoff,
                                                         w.rot_abc[0], w.rot_abc[1], w.rot_abc[2], w.rn_ratio))
    if w.worm is not None:
        lines.append("WORM %s %r %d" % (w.worm[0], float(w.worm[1]), int(w.worm[2])))
    lines += ["NUMBEROFSLICES %d" % w.nslices, "NUMBEROFPASSES %d" % passes,
              "NUMBEROFBLOCKS %d 0" % blocks, "MCSKIP_RATIO 1000000", "MCSKIP_TOTAL 1000000", "MCSKIP_AVERG 1"]
    with open(os.path.join(workdir, "qmc.input"), "w") as f:
        f.write("\n".join(lines) + "\n")
    tb = w.tables
    for t in w.types:
        if t["molecule"] == 0 and "grid1d" in tb:
            with open(os.path.join(workdir, t["fpot"] + ".pot"), "w") as f:
                f.write("# synthetic 1D potential (A, K)\n")
                for r, v in zip(tb["grid1d"], tb["pot1d"]):
                    f.write("%.17g %.17g\n" % (r, v))
        if t["molecule"] == 1 and "pot2d" in tb:
            rg, cg, v = tb["rgrid2d"], tb["cgrid2d"], tb["pot2d"]
            with open(os.path.join(workdir, t["fpot"] + ".pot"), "w") as f:
                f.write("%d %d\n%.17g %.17g\n" % (len(rg), len(cg), tb["dr2d"], tb["dc2d"]))
                f.write("\n".join("%.17g" % x for x in rg) + "\n")
                f.write("\n".join("%.17g" % x for x in cg) + "\n")
                f.write("\n".join("%.17g" % x for x in v.ravel()) + "\n")
            rname = "%s_T%st%d.rot" % (t["name"], _fmt_temperature(w.temperature), w.nrotslices)
            with open(os.path.join(workdir, rname), "w") as f:
                for row in zip(tb["rotgrid"], tb["rotdens"], tb["rotderv"], tb["rotesqr"]):
                    f.write(" ".join("%.17g" % x for x in row) + "\n")
