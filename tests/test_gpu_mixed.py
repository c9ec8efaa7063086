"""The FP32 table path (pimc_set_precision(h, 1)): pair terms, table
densities and rattle-and-shake log-densities in float from float copies of
beads, frames and tables; sums, action differences and the tests in FP64.
Checked move by move against the FP64 oracle on the
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
    """Every move of the fixture's sequence is compared.  Where a decision
    differs (the uniform lies within the FP32 tolerance of the acceptance
    probability), the quantity it was made from must still agree within the
    tolerance; the GPU path is then set to the oracle's and the sequence goes
    on, so no move is left out.  Such resynchronisations must stay rare."""
    w, d, _ = golden(name)
    s = G.Sampler(w, mixed=True)
    o = O.Oracle(w)
    st = split_streams(d)
    tau = 1.0 / (w.temperature * w.nslices)
    emax = float(np.max(np.abs(d["e_slice"])))
    erot = float(np.max(np.abs(d["e_rot"]))) if w.rotation else 0.0
    R = w.nslices // w.nrotslices
    ib = im = ir = 0
    compared = parted = 0

    def resync():
        c, a, _, p = o.get_state()
        s.set_state(c, a, p)

    for kind, typ, t in d["seq"]:
        typ, t = int(typ), int(t)
        if kind == 0:
            g, u3 = st["gauss"][ib], st["u3"][ib]; ib += 1
            rs, ds, lv, cons = s.bisection_move(typ, t, g, u3)
            _, ods, olv, ocons = o.bisection_move(typ, t, g, u3)
            assert rs == 0
            M = 1 << w.types[typ]["levels"]
            tol = RTOL32 * np.maximum(np.abs(ods), tau * M * M * emax)
            lvc = np.minimum(lv, olv)          # levels both reached
            mask = np.arange(ds.shape[1])[None, :] <= np.minimum(lvc, ds.shape[1] - 1)[:, None]
            # atoms after the first differing decision move on different paths
            k = int(np.argmax(lv != olv)) if not (lv == olv).all() else len(lv)
            mask[k + 1:] = False
            assert (np.abs(ds - ods)[mask] <= tol[mask]).all(), (ds, ods)
            if not (lv == olv).all():
                parted += 1
                resync()
            else:
                assert cons == ocons
        elif kind == 1:
            u1, u2 = st["u1"][im], st["u2"][im]; im += 1
            rs, dv, acc, cons = s.molecular_move(typ, u1, u2)
            _, odv, oacc, ocons = o.molecular_move(typ, u1, u2)
            assert rs == 0
            k = int(np.argmax(acc != oacc)) if not (acc == oacc).all() else len(acc)
            # atoms up to the first differing decision read identical paths
            sc = RTOL32 * np.maximum(np.abs(odv), 2 * w.nslices * emax)
            assert (np.abs(dv - odv)[:k + 1] <= sc[:k + 1]).all()
            if k < len(acc):
                parted += 1
                resync()
        else:
            ur = st["urot"][ir]; ir += 1
            rs, rd, acc = s.rotations(ur)
            _, ord_, oacc, _ = o.rotations(typ, ur)
            assert rs == 0
            scale = np.maximum(np.abs(ord_), 1.0) * max(1.0, tau * 2 * R * erot)
            if not (acc == oacc).all():
                k = int(np.argmax(acc != oacc))
                assert (np.abs(rd - ord_)[:k + 1] <= RTOL32 * scale[:k + 1]).all()
                parted += 1
                resync()
            else:
                assert (np.abs(rd - ord_) <= RTOL32 * scale).all(), np.max(np.abs(rd - ord_) / scale)
        compared += 1
    assert compared == len(d["seq"])
    assert parted <= max(1, len(d["seq"]) // 10), (parted, compared)
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
