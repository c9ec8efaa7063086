"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own C++ (compiled from its sources into oracle/_ref by
oracle/ref_build.sh, Fortran leaves bound to the oracle's C restatements)
on small seeded systems of the three benchmark families, with replayed
random numbers, and stores inputs and outputs:

  * PotEnergy per slice / whole path (mc_piqmc.cc:1201-1383,1796-1965),
    PotRotEnergy / PotRotE3D (mc_piqmc.cc:1967-2151) on given configurations;
  * a sequence of MCBisectionMove, MCMolecularMove and MCRotationsMove /
    MCRotations3D calls (mc_piqmc.cc:54-1199): the final path, the accept
    counters and the number of random numbers each generator consumed;
  * the worm branch of the pass loop on a small He-4 system (c0w): MCWormMove
    calls (mc_qworm.cc:93-125) and, with the worm closed,
    MCBisectionMoveExchange and MCMolecularMoveExchange under the
    permutations the swaps build;
  * the estimators GetKinEnergy, GetPotEnergy_Densities, GetRotEnergy /
    GetRotE3D (mc_estim.cc:500-1096) of the final path;
  * with bosons, under a random permutation: the density histograms of
    GetPotEnergy_Densities (non-zero bins only), GetExchangeLength,
    GetAreaEstimators and GetAreaEstim3D in both frames
    (mc_estim.cc:1233-1286, 1997-2594).

The reference runs single-threaded: its whole-path PotEnergy shares one
dr[3] array across OpenMP threads (mc_piqmc.cc:1210,1237) and is not
reproducible with more than one thread.  Tables are regenerated from the
seeds at test time (workloads.py), so only their checksums are stored.

Usage (here, where the reference tree exists):
    oracle/ref_build.sh && OMP_NUM_THREADS=1 python tests/golden/make_golden.py
"""
import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "moribs-pimc_gb300"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
import workloads as W  # noqa: E402

CASES = {
    "c0s": ("config0", dict(seed=11, nslices=32, nrotslices=8, n_he=4, r2d_step=0.05, c2d_step=0.04)),
    "c1s": ("config1", dict(seed=12, nslices=32, nrotslices=8, n_h2=6, grid3d=(30, 37, 19), griddens=(19, 37, 37))),
    "c3s": ("config3", dict(seed=13, nslices=64, nrotslices=16, griddens=(19, 37, 37))),
    # the rattle-and-shake propagator (ROTDENSI 1, rotden.f:218-286) in the moves
    "c3r": ("config3", dict(seed=14, nslices=64, nrotslices=16, griddens=(19, 37, 37), rot_den_type=1)),
    # the water-chain family: 3 waters (caleng between them) + 4 pH2 (vcord), ROTDENSI 1
    "c4s": ("water_chain_case", dict(seed=16, nrot=3, nh2=4, nslices=32, nrotslices=8, T=1.2,
                                     griddens=(19, 37, 37))),
    # ISPHER = 1: vspher for the rotor-pH2 terms of the translational moves
    # (vspher.f); the reference allows it only without rotation (mc_input.cc)
    "c1p": ("config1", dict(seed=15, nslices=32, nrotslices=8, n_h2=6, grid3d=(30, 37, 19), griddens=(19, 37, 37),
                            ispher=1), dict(rotation=False)),
}


def make_workload(case):
    fn, kw = CASES[case][:2]
    w = getattr(W, fn)(**kw)
    for k, v in (CASES[case][2] if len(CASES[case]) > 2 else {}).items():
        setattr(w, k, v)
    return w


def table_checksums(w):
    out = {}
    for k, v in sorted(w.tables.items()):
        if isinstance(v, np.ndarray):
            out["tab_" + k] = np.array([float(np.sum(v)), float(np.sum(np.abs(v))), float(v.ravel()[len(v.ravel()) // 3])])
    return out


def generate(case, nsteps=4, seed=2024):
    w = make_workload(case)
    rng = np.random.default_rng(seed)
    ref = O.Reference(w)
    nb = w.natoms * w.nslices
    res = dict(case=np.array(case), coords0=w.coords.copy(), angles0=w.angles.copy())
    res.update(table_checksums(w))
    c0 = np.ascontiguousarray(w.coords)
    # ---- energies on the initial path and on a displaced path
    pos = np.ascontiguousarray(c0 + rng.normal(0.0, 0.05, c0.shape))
    slices = np.array([0, 3, w.nslices // 2, w.nslices - 1], dtype=np.int32)
    e_slice = np.zeros((w.natoms, len(slices), 2))
    e_path = np.zeros((w.natoms, 2))
    for a in range(w.natoms):
        for j, it in enumerate(slices):
            e_slice[a, j, 0] = ref.L.ref_pot_energy_slice(a, O.dptr(c0), int(it))
            e_slice[a, j, 1] = ref.L.ref_pot_energy_slice(a, O.dptr(pos), int(it))
        e_path[a, 0] = ref.L.ref_pot_energy_path(a, O.dptr(c0))
        e_path[a, 1] = ref.L.ref_pot_energy_path(a, O.dptr(pos))
    res.update(pos=pos, slices=slices, e_slice=e_slice, e_path=e_path)
    # rotor energies: random orientation sets
    rot_types = [i for i, t in enumerate(w.types) if t["molecule"] != 0]
    rtype = rot_types[0]
    roff = sum(t["numb"] for t in w.types[:rtype])
    eul = np.column_stack([rng.uniform(0, 2 * np.pi, 6), np.arccos(rng.uniform(-1, 1, 6)), rng.uniform(0, 2 * np.pi, 6)])
    e_rot = np.zeros((6, len(slices)))
    cosine = None
    if not w.rotation:
        pass                              # no PotRotE3D / PotRotEnergy calls without rotation
    elif w.types[rtype]["molecule"] == 1:
        cosine = np.zeros((3, nb))
        for k in range(6):
            cosine[:, :] = 0.0
            th, ph = eul[k, 1], eul[k, 0]
            cosine[0, :] = np.sin(th) * np.cos(ph)
            cosine[1, :] = np.sin(th) * np.sin(ph)
            cosine[2, :] = np.cos(th)
            cz = np.ascontiguousarray(cosine)
            for j, it in enumerate(slices):
                e_rot[k, j] = ref.L.ref_pot_rot_energy(roff, O.dptr(cz), int(it))
    else:
        for k in range(6):
            e = np.ascontiguousarray(eul[k])
            for j, it in enumerate(slices):
                e_rot[k, j] = ref.L.ref_pot_rot_e3d(roff, O.dptr(e), int(it))
    res.update(eul=eul, e_rot=e_rot)
    # ---- a move sequence with replayed randoms
    seq = []
    streams = dict(gauss=[], u1=[], u2=[], u3=[], urot=[])
    consumed = []
    times = rng.integers(0, w.nslices, size=nsteps * len(w.types))
    k = 0
    for step in range(nsteps):
        for typ in range(len(w.types)):
            g = rng.normal(size=3 * w.types[typ]["numb"] * (1 << w.types[typ]["levels"]))
            u3 = rng.uniform(size=w.types[typ]["numb"] * w.types[typ]["levels"])
            t = int(times[k]); k += 1
            ref.replay(gauss=g, u3=u3)
            ref.L.ref_bisection_move(typ, t)
            consumed.append(ref.replay_pos())
            seq.append((0, typ, t))
            streams["gauss"].append(g); streams["u3"].append(u3)
        for typ in range(len(w.types)):
            n = w.types[typ]["numb"]
            u1 = rng.uniform(size=3 * n); u2 = rng.uniform(size=n)
            ref.replay(u1=u1, u2=u2)
            ref.L.ref_molecular_move(typ)
            consumed.append(ref.replay_pos())
            seq.append((1, typ, 0))
            streams["u1"].append(u1); streams["u2"].append(u2)
        if not w.rotation:
            continue
        nr = w.types[rtype]["numb"]
        ur = rng.uniform(size=4 * w.nrotslices * nr)
        ref.replay(urot=ur)
        if w.types[rtype]["molecule"] == 1:
            ref.L.ref_rotations_move(rtype)
        else:
            ref.L.ref_rotations_3d(rtype)
        consumed.append(ref.replay_pos())
        seq.append((2, rtype, 0))
        streams["urot"].append(ur)
    c, a, co = ref.get_state()
    tot, acc = ref.counters()
    # IOxyz's file of the final path (mc_input.cc:690-794), as text
    xyzf = os.path.join(ref.tmp, "final.xyz")
    ref.L.ref_write_xyz(xyzf.encode())
    with open(xyzf) as f:
        res["xyz_text"] = np.array(f.read())
    res.update(seq=np.array(seq, dtype=np.int32), consumed=np.array(consumed, dtype=np.int64),
               coords1=c, angles1=a, cosine1=co, total=tot, accep=acc)
    for name, lst in streams.items():
        res["s_" + name] = np.concatenate(lst) if lst else np.zeros(0)
        res["n_" + name] = np.array([len(x) for x in lst], dtype=np.int64)
    # ---- estimators on the final path
    kin = ref.L.ref_kin_energy()
    esq, ets = np.zeros(1), np.zeros(1)
    if not w.rotation:
        rot = 0.0
    elif w.types[rtype]["molecule"] == 1:
        rot = ref.L.ref_rot_energy(O.dptr(esq), O.dptr(ets))
    else:
        rot = ref.L.ref_rot_e3d(O.dptr(esq), O.dptr(ets))
    pot = ref.L.ref_pot_energy_est()
    res.update(est=np.array([kin, pot, rot, esq[0], ets[0]]))
    # ---- densities, exchange cycles and area estimators of the final path
    # under a permutation of the bosons (mc_estim.cc:500-687, 1997-2594)
    bos = [i for i, t in enumerate(w.types) if t["stat"] == 1]
    if bos:
        nbos = w.types[bos[-1]]["numb"]
        perm = np.arange(w.natoms, dtype=np.int32)
        perm[:nbos] = rng.permutation(nbos)
        ref.set_pindex(perm)
        v, g1, g2, g3 = ref.densities()
        res.update(perm=perm, dens_pot=np.array(v), masses=np.array([ref.L.ref_mass(t) for t in range(len(w.types))]))
        for k, g in (("g1", g1), ("g2", g2), ("g3", g3)):
            flat = g.ravel()
            nz = np.flatnonzero(flat)
            res["dens_%s_idx" % k] = nz.astype(np.int64)
            res["dens_%s_cnt" % k] = flat[nz]
        res["ploops"] = ref.exchange_lengths(nbos)
        if w.types[rtype]["molecule"] == 1:
            res["area2d"] = ref.area_estimators()
        res["area3d"] = np.stack([ref.area_estim3d(0), ref.area_estim3d(1)])
    return res


WORM_CASE = dict(seed=21, nslices=32, nrotslices=8, n_he=6, r2d_step=0.05, c2d_step=0.04)
WORM_LINE = ("He4", 2.0, 6)


def make_worm_workload():
    w = W.config0(**WORM_CASE)
    w.worm = WORM_LINE
    return w


def generate_worm(ncalls=40, seed=77):
    """The worm branch of the pass loop (mc_main.cc:356-379): MCWormMove, and
    while the worm is closed an MCBisectionMoveExchange of the boson type at
    a drawn slice (a window inside the ring) and an MCMolecularMoveExchange, on 6 He-4 around the linear rotor, P = 32, WORM He4 2.0 6.
    Per call: the replayed streams, the draws consumed, the worm state; at the
    end the path, the permutation and the worm counters."""
    w = make_worm_workload()
    rng = np.random.default_rng(seed)
    ref = O.Reference(w)
    nbos = w.types[0]["numb"]
    res = dict(case=np.array("c0w"), coords0=w.coords.copy(), angles0=w.angles.copy())
    streams = {n: [] for n in O.WSTREAMS}
    cons, states, seq, bis = [], [], [], dict(gauss=[], u3=[], t=[], cons=[])
    for k in range(ncalls):
        st = {n: rng.uniform(1e-6, 1.0 - 1e-6, 4 * nbos) for n in O.WSTREAMS if n != "gauss"}
        st["gauss"] = rng.normal(0.0, 1.0 / np.sqrt(2.0), 3 * nbos * (3 * WORM_LINE[2] + 8))
        for n in O.WSTREAMS:
            streams[n].append(st[n])
        cons.append(ref.worm_move(st)[:9])
        states.append(ref.worm_state())
        if not states[-1][0]:
            # windows that do not cross the end of the ring: across it the
            # reference evaluates the wrong atom's bead (mc_piqmc.cc:373-376)
            t = int(rng.integers(0, w.nslices - (1 << w.types[0]["levels"])))
            g = rng.normal(0.0, 1.0 / np.sqrt(2.0), 3 * nbos * 8)
            u3 = rng.uniform(size=nbos * 3)
            ref.replay(u3=u3, gauss=g)
            ref.L.ref_bisection_move_exchange(0, t)
            pos = ref.replay_pos()
            bis["gauss"].append(g); bis["u3"].append(u3); bis["t"].append(t); bis["cons"].append((pos[3], pos[2]))
            seq.append((k, len(bis["t"]) - 1))
            # MCMolecularMoveExchange (mc_main.cc:371-377), one displacement per cycle
            u1 = rng.uniform(size=3 * nbos)
            u2 = rng.uniform(size=nbos)
            ref.replay(u1=u1, u2=u2)
            ref.L.ref_molecular_move_exchange(0)
            pos = ref.replay_pos()
            bis.setdefault("u1", []).append(u1); bis.setdefault("u2", []).append(u2)
            bis.setdefault("mcons", []).append((pos[0], pos[1]))
    c, a, co = ref.get_state()
    p, r = ref.pindex()
    tot, acc = ref.worm_counters()
    for n in O.WSTREAMS:
        res["w_" + n] = np.concatenate(streams[n])
        res["wn_" + n] = np.array([len(x) for x in streams[n]], dtype=np.int64)
    res.update(w_consumed=np.array(cons, dtype=np.int64), w_states=np.array(states, dtype=np.int32),
               w_bis_after=np.array(seq, dtype=np.int32).reshape(-1, 2), w_bis_t=np.array(bis["t"], dtype=np.int32),
               w_bis_gauss=np.concatenate(bis["gauss"]) if bis["gauss"] else np.zeros(0),
               w_bis_u3=np.concatenate(bis["u3"]) if bis["u3"] else np.zeros(0),
               w_bis_cons=np.array(bis["cons"], dtype=np.int64).reshape(-1, 2),
               w_mol_u1=np.concatenate(bis["u1"]), w_mol_u2=np.concatenate(bis["u2"]),
               w_mol_cons=np.array(bis["mcons"], dtype=np.int64).reshape(-1, 2),
               coords1=c, angles1=a, pindex1=p, rindex1=r, w_total=tot[[0, 1, 4, 5, 6]], w_accep=acc[[0, 1, 4, 5, 6]])
    return res


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/libref.so missing: run oracle/ref_build.sh first")
    for case in CASES:
        res = generate(case)
        path = os.path.join(HERE, case + ".npz")
        np.savez_compressed(path, **res)
        print("wrote", path, os.path.getsize(path), "bytes")
    res = generate_worm()
    path = os.path.join(HERE, "c0w.npz")
    np.savez_compressed(path, **res)
    print("wrote", path, os.path.getsize(path), "bytes", "worm states", res["w_states"][:, 0].tolist(),
          "bisections", len(res["w_bis_t"]), "swaps accepted", res["w_accep"][4])


if __name__ == "__main__":
    main()
