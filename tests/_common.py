"""Shared helpers for the tests: fixtures, replay of golden move sequences."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_golden(case):
    import make_golden as M  # tests/golden is on sys.path via load below
    return M


def golden_cases():
    return ["c0s", "c1s", "c3s", "c3r", "c4s", "c1p"]


def nrotors(w):
    return sum(t["numb"] for t in w.types if t["molecule"] != 0)


def rot_est_from_reference(w):
    """Which rotational estimators of the fixture (est[2], est[3..4]) the
    reference computes as intended.  GetRotE3D advances the rotor offset
    cumulatively (mc_estim.cc:1000-1003), so with three or more rotors it
    reads past the rotors' angles; with the rattle-and-shake density it
    converts the running sum of all rotors once per rotor
    (mc_estim.cc:1084-1090), so E_rot of two or more rotors is not their
    sum.  Those values are compared with the oracle, which keeps each rotor
    at its own offset and converts each rotor's sum once."""
    n = nrotors(w) if w.rotation else 0
    erot_ok = n <= 1 or (n == 2 and w.rot_den_type == 0)
    sq_ok = n <= 2
    return erot_ok, sq_ok


def rs_rotor_means(w, angles):
    """Per rotor, the mean over its Q links of rsrot's rho (the
    rattle-and-shake exponent sumaxs, rotden.f:247-284) from the reference's
    angle array (phi, cos theta, chi)."""
    import workloads as W
    P, Q = w.nslices, w.nrotslices
    rt = [i for i, t in enumerate(w.types) if t["molecule"] != 0][0]
    first = sum(t["numb"] for t in w.types[:rt])
    bl = 1.0 / np.asarray(w.rot_abc, dtype=np.float64)
    out = []
    for r in range(w.types[rt]["numb"]):
        a = (first + r) * P
        ph, ct, ch = angles[0, a:a + Q], angles[1, a:a + Q], angles[2, a:a + Q]
        m = W.matpre(ph, np.arccos(ct), ch)                       # [3][3][Q]
        m2 = np.roll(m, -1, axis=2)
        dig = [np.sum(m[:, i, :] * m2[:, i, :], axis=0) for i in range(3)]
        sumaxs = ((bl[0] - bl[1] - bl[2]) * (1.0 - dig[0]) + (bl[1] - bl[2] - bl[0]) * (1.0 - dig[1])
                  + (bl[2] - bl[0] - bl[1]) * (1.0 - dig[2]))
        out.append(float(np.mean(sumaxs)))
    return out


def rs_energy(w, mean_sumaxs):
    """GetRotE3D's rattle-and-shake conversion of a link mean (mc_estim.cc:1084-1090), K."""
    wno2k = 0.6950356
    tau = 1.0 / (w.temperature * w.nrotslices) / wno2k
    e = mean_sumaxs / (4.0 * tau * tau) + 0.25 * float(np.sum(w.rot_abc)) + 1.5 / tau
    return e / wno2k


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


def dense_hist(d, key, shape):
    """A histogram stored as non-zero bins (dens_<key>_idx/_cnt) back to shape."""
    out = np.zeros(int(np.prod(shape)))
    out[d["dens_%s_idx" % key]] = d["dens_%s_cnt" % key]
    return out.reshape(shape)


def area_scales(w, coords, masses):
    """Magnitude bounds of the area-estimator sums of one path: s_area bounds
    sum |n . (dr0 x dr1)| / 2 over beads, s_inert sum |(n x dr0).(n x dr1)| m / P."""
    nbos = [t["numb"] for t in w.types if t["stat"] == 1][-1]
    c = np.asarray(coords).reshape(3, w.natoms, w.nslices)
    span = np.max(np.linalg.norm(c - c.mean(axis=1, keepdims=True), axis=0)) * 2.0
    s_area = nbos * w.nslices * span * span
    return s_area, nbos * span * span * max(1.0, float(np.max(masses)))


def check_area(got, ref, s_area, s_inert, three_d, rtol=1e-10):
    """Area-estimator outputs against the reference's: sums within rtol of
    their magnitude bound, products of two sums within rtol of s_area times
    the two sums' sizes."""
    got, ref = np.asarray(got, float), np.asarray(ref, float)
    if three_d:      # area_proj[3] (GPU/oracle only), products[6], inert[9]
        a = got[:3]
        pairs = [(i, j) for i in range(3) for j in range(i + 1)]
        ps = np.array([s_area * (abs(a[i]) + abs(a[j])) + s_area * s_area * rtol for i, j in pairs])
        g, r = got[3:], ref
        scale = np.concatenate([ps, np.full(9, s_inert)])
    else:            # areas[2], area2[2], inert[2]
        a = got[:2]
        scale = np.array([s_area, s_area, 2 * s_area * abs(a[0]) + s_area * s_area * rtol,
                          2 * s_area * abs(a[1]) + s_area * s_area * rtol, s_inert, s_inert])
        g, r = got, ref
    err = np.abs(g - r)
    assert np.all(err <= rtol * scale), "area estimators: err/scale %s" % (err / scale)
