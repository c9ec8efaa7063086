"""Full runs against the oracle: the GPU's production passes (checkerboard
slices, independent sets, Philox draws) and the oracle's restatement of the
reference schedule (serial slices, its own draws) sample the same
distribution, so their estimators agree within the combined standard error
of block means (mc_estim.cc:500-1096 estimators, sampled once per pass as
mc_main.cc:551-616 does)."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu

NAMES = ("E_kin", "E_pot", "E_rot", "<cos gamma(beta/2)>")


def _blocks(sample, nblocks, per):
    out = np.zeros((nblocks, len(NAMES)))
    for b in range(nblocks):
        for _ in range(per):
            out[b] += sample()
        out[b] /= per
    return out


def test_production_runs_agree_with_the_oracle_within_standard_errors():
    """Config 0 shape at a small size (linear rotor + 4 He, P = 64, Q = 16):
    500 equilibration passes, then 40 blocks of 50 passes on each side.
    The acceptance bound is 3 combined standard errors per estimator (four
    estimators are tested at once; 2 would fail by chance in about one run
    of six)."""
    w = W.config0(seed=5, nslices=64, nrotslices=16, n_he=4)
    nb, per, equil = 40, 50, 500
    # the orientational estimator: GetRCF's <cos gamma> between the rotor's
    # axis at two slices half a period apart, averaged over the time origins
    # (mc_estim.cc:1099-1139 sums over the Q origins).  The
    # lab-frame <cos theta> is no test here: with no field it relaxes from the
    # initial orientation over far more passes than the run has.
    half = w.nrotslices // 2
    s = G.Sampler(w)
    s.run_passes(equil, seed=11)

    def gpu():
        s.run_passes(1, seed=11)
        return np.append(s.estimators()[:3], s.rcf()[half] / w.nrotslices)
    g = _blocks(gpu, nb, per)
    s.close()
    o = O.Oracle(w)
    state = {"p": 0}

    def step():
        st, _ = o.run_steps(0, w.nslices, seed=70000 + state["p"])
        assert st == 0
        state["p"] += 1
    for _ in range(equil):
        step()

    def cpu():
        step()
        return np.array([o.kin_energy(), o.pot_energy_est(), o.rot_energy(False)[0], o.rcf()[half] / w.nrotslices])
    c = _blocks(cpu, nb, per)
    mg, mc = g.mean(0), c.mean(0)
    se = np.hypot(g.std(0, ddof=1), c.std(0, ddof=1)) / np.sqrt(nb)
    z = (mg - mc) / se
    report = {n: (round(a, 4), round(b, 4), round(e, 4), round(zz, 2)) for n, a, b, e, zz in zip(NAMES, mg, mc, se, z)}
    print("block means (GPU, oracle, combined SE, z):", report)
    assert np.all(np.isfinite(z)), report
    assert np.all(np.abs(z) <= 3.0), report
