"""The FP32 table path (pimc_set_precision(h, 1)): pair terms in float from
float copies of beads and tables, sums, action differences, exponentials and
densities in FP64.  Checked move by move against the FP64 oracle on the
reference-generated move sequences: action differences and acceptance
ratios within 1e-5 of the energy terms they are built from, and the same
accept decisions unless the uniform lies within that tolerance of the
acceptance probability (then the paths may legitimately part and the
comparison stops)."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
from _common import golden, golden_cases, split_streams

pytestmark = pytest.mark.gpu
RTOL32 = 1e-5


@pytest.mark.parametrize("name", golden_cases())
def test_mixed_precision_moves_track_the_fp64_oracle(name):
    w, d, _ = golden(name)
    s = G.Sampler(w, mixed=True)
    o = O.Oracle(w)
    st = split_streams(d)
    tau = 1.0 / (w.temperature * w.nslices)
    emax = float(np.max(np.abs(d["e_slice"])))
    erot = float(np.max(np.abs(d["e_rot"])))
    R = w.nslices // w.nrotslices
    ib = im = ir = 0
    compared = 0
    for kind, typ, t in d["seq"]:
        typ, t = int(typ), int(t)
        if kind == 0:
            g, u3 = st["gauss"][ib], st["u3"][ib]; ib += 1
            rs, ds, lv, cons = s.bisection_move(typ, t, g, u3)
            _, ods, olv, ocons = o.bisection_move(typ, t, g, u3)
            assert rs == 0
            M = 1 << w.types[typ]["levels"]
            tol = RTOL32 * np.maximum(np.abs(ods), tau * M * M * emax)
            if not (lv == olv).all():
                break                      # a borderline level decision: paths part here
            mask = np.arange(ds.shape[1])[None, :] <= np.minimum(lv, ds.shape[1] - 1)[:, None]
            assert (np.abs(ds - ods)[mask] <= tol[mask]).all(), (ds, ods)
            assert cons == ocons
        elif kind == 1:
            u1, u2 = st["u1"][im], st["u2"][im]; im += 1
            rs, dv, acc, cons = s.molecular_move(typ, u1, u2)
            _, odv, oacc, ocons = o.molecular_move(typ, u1, u2)
            assert rs == 0
            assert (np.abs(dv - odv) <= RTOL32 * np.maximum(np.abs(odv), 2 * w.nslices * emax)).all()
            if not (acc == oacc).all():
                break
        else:
            ur = st["urot"][ir]; ir += 1
            rs, rd, acc = s.rotations(ur)
            _, ord_, oacc, _ = o.rotations(typ, ur)
            assert rs == 0
            scale = np.maximum(np.abs(ord_), 1.0) * max(1.0, tau * 2 * R * erot)
            if not (acc == oacc).all():
                k = int(np.argmax(acc != oacc))
                assert abs(rd[k] - ord_[k]) <= RTOL32 * scale[k]
                break
            assert (np.abs(rd - ord_) <= RTOL32 * scale).all(), np.max(np.abs(rd - ord_) / scale)
        compared += 1
    assert compared >= 3
    s.close()


def test_mixed_precision_production_pass_runs():
    w, d, _ = golden("c1s")
    s = G.Sampler(w, mixed=True)
    s.run_passes(3, seed=5)
    s.synchronize()
    tot, acc = s.counters()
    assert tot[1] == 3 * w.types[0]["numb"] * w.nslices
    c, a, co, _ = s.get_state()
    assert np.isfinite(c).all() and np.isfinite(a).all()
    s.close()
