"""Golden fixtures for the propagator-table generators, taken from the
outputs the reference ships (read as text, written by its own generators):

  * examples/CO2_100K_4_4/CO2_T100t4.rot and
    examples/N2O_5pH2_0.5K_512_128/N2O_T0.5t128.rot -- linden.f tables
    (T = 100 K, 4 slices, 3000 points; T = 0.5 K, 128 slices, 1400 points).
    Their rotational constants are not recorded with them; B = 0.39021 and
    0.419 cm^-1 reproduce them to the 8 significant digits they carry;
  * nmv_prop/rho.den010_{rho,eng,esq} -- the theta = 10 degree slab of
    asymrho.f for the run in nmv_prop/a-run (T = 0.37 K, 128 slices,
    iodevn -1, A B C = 0.6666525 0.2306476 0.1769383 cm^-1, maxj 66), a
    seeded subset of 4000 of its 361*361 points, and the "AT BETA" / "AT
    TAU" partition-function lines and the j <= 2 eigenvalues of nmv_prop/log.

Usage (where the reference tree exists):
    python tests/golden/make_tables_golden.py REFERENCE_DIR
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: the first argument, else PIMC_REFERENCE_DIR
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PIMC_REFERENCE_DIR", "")
if not REF or not os.path.isdir(REF):
    sys.exit("usage: make_tables_golden.py REFERENCE_DIR (or set PIMC_REFERENCE_DIR)")


def main():
    out = {}
    for key, rel, T, ns, B in (("co2", "examples/CO2_100K_4_4/CO2_T100t4.rot", 100.0, 4, 0.39021),
                               ("n2o", "examples/N2O_5pH2_0.5K_512_128/N2O_T0.5t128.rot", 0.5, 128, 0.419)):
        d = np.loadtxt(os.path.join(REF, rel))
        rows = np.arange(0, len(d), 3)
        out["linden_%s_rows" % key] = rows
        out["linden_%s_table" % key] = d[rows]
        out["linden_%s_params" % key] = np.array([T, ns, B, len(d)])
    slab = [np.loadtxt(os.path.join(REF, "nmv_prop", "rho.den010_" + k)) for k in ("rho", "eng", "esq")]
    rng = np.random.default_rng(10)
    idx = np.sort(rng.choice(361 * 361, 4000, replace=False))
    out["asym_idx"] = idx
    out["asym_vals"] = np.stack([s[idx] for s in slab])
    out["asym_maxabs"] = np.array([np.max(np.abs(s)) for s in slab])
    out["asym_params"] = np.array([0.37, 128, -1, 10, 0.6666525, 0.2306476, 0.1769383, 66])
    log = open(os.path.join(REF, "nmv_prop", "log")).read()
    nums = []
    for tag in ("AT BETA", "AT TAU"):
        blk = log.split(tag, 1)[1].split("\n")[1:4]
        for line in blk:
            v = [float(x) for x in re.findall(r"=\s*([-0-9.Ee+]+)", line)]
            nums += [v[0], v[1]] + ([v[3]] if tag == "AT BETA" else [])   # Z, E (cm^-1)[, Cv]
    out["asym_info"] = np.array(nums)
    # eigenvalues of the j <= 2 blocks printed after each rotational matrix
    ev = []
    for chunk in log.split("rotational matrix for ")[1:]:
        lines = [ln for ln in chunk.split("\n")[1:] if ln.strip()]
        n = len(lines[0].split())
        ev += [float(x) for x in lines[n].split()]
    out["asym_log_eigs"] = np.array(sorted(ev))
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **out)
    print("wrote", os.path.join(HERE, "tables.npz"), os.path.getsize(os.path.join(HERE, "tables.npz")))


if __name__ == "__main__":
    main()
