"""Full runs against the oracle: the GPU's production passes (checkerboard
slices, independent sets, Philox draws) and the oracle's restatement of the
reference schedule (serial slices, its own draws) sample the same
distribution, so their estimators agree within two combined standard errors
of block means (mc_estim.cc:500-1096 estimators, sampled once per pass as
mc_main.cc:551-616 does), in both precisions of the GPU path.

Systems (reduced slices and particle counts, so that the serial oracle
finishes in seconds): the config-0 shape (linear rotor + 4 He, P = 64,
Q = 16), the config-1 shape (asymmetric top + 6 pH2, P = 64, Q = 16, 3D
rotor-pH2 table and top density of the c1s fixture grids) and the config-3
shape (water dimer, caleng, P = 64, Q = 32).  Seeds are fixed, and the GPU
passes and the oracle are both deterministic, so the test is reproducible.

Estimators: E_kin, E_pot, E_rot and the orientational correlation
<cos gamma(beta/2)> of GetRCF between rotational slices half a period apart
(mc_estim.cc:1099-1139); the lab-frame <cos theta> relaxes from the initial
orientation over far more passes than a run has (no field), so the rotor's
orientation enters through the correlation."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu

NAMES = ("E_kin", "E_pot", "E_rot", "<cos gamma(beta/2)>")
SYSTEMS = {
    "config0": lambda: W.config0(seed=5, nslices=64, nrotslices=16, n_he=4),
    "config1": lambda: W.config1(seed=6, nslices=64, nrotslices=16, n_h2=6, grid3d=(30, 37, 19),
                                 griddens=(19, 37, 37)),
    "config3": lambda: W.config3(seed=7, nslices=64, nrotslices=32, griddens=(19, 37, 37), levels=3),
}
NB, PER, EQUIL = 40, 50, 500
_oracle_cache = {}


def _blocks(sample, nblocks, per):
    out = np.zeros((nblocks, len(NAMES)))
    for b in range(nblocks):
        for _ in range(per):
            out[b] += sample()
        out[b] /= per
    return out


def _oracle_blocks(name):
    if name in _oracle_cache:
        return _oracle_cache[name]
    w = SYSTEMS[name]()
    half = w.nrotslices // 2
    nonlinear = any(t["molecule"] == 2 for t in w.types)
    o = O.Oracle(w)
    state = {"p": 0}

    def step():
        st, _ = o.run_steps(0, w.nslices, seed=70000 + state["p"])
        assert st == 0
        state["p"] += 1
    for _ in range(EQUIL):
        step()

    def cpu():
        step()
        return np.array([o.kin_energy(), o.pot_energy_est(), o.rot_energy(nonlinear)[0], o.rcf()[half] / w.nrotslices])
    _oracle_cache[name] = _blocks(cpu, NB, PER)
    return _oracle_cache[name]


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name", list(SYSTEMS))
def test_production_runs_agree_with_the_oracle_within_two_standard_errors(name, mixed):
    w = SYSTEMS[name]()
    half = w.nrotslices // 2
    s = G.Sampler(w, mixed=mixed)
    s.run_passes(EQUIL, seed=11)

    def gpu():
        s.run_passes(1, seed=11)
        return np.append(s.estimators()[:3], s.rcf()[half] / w.nrotslices)
    g = _blocks(gpu, NB, PER)
    s.close()
    c = _oracle_blocks(name)
    mg, mc = g.mean(0), c.mean(0)
    se = np.hypot(g.std(0, ddof=1), c.std(0, ddof=1)) / np.sqrt(NB)
    z = (mg - mc) / se
    report = {n: (round(a, 5), round(b, 5), round(e, 5), round(zz, 2)) for n, a, b, e, zz in zip(NAMES, mg, mc, se, z)}
    print("%s %s block means (GPU, oracle, combined SE, z):" % (name, "fp32" if mixed else "fp64"), report)
    assert np.all(np.isfinite(z)), report
    assert np.all(np.abs(z) <= 2.0), report
