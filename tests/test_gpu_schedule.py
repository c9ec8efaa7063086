"""The production schedule's fused kernels against the phase-by-phase
launches: a bisection block runs the numb phases of one (type, s0) in one
launch, and the persistent rotational kernel runs many half-sweeps with
neighbour-to-neighbour waits.  Both read exactly the state the one-launch-
per-phase schedule reads, with the same uniforms, so the paths after a pass
must be bit-identical.  Also the odd-Q rotational sweep, where the last even
slice neighbours slice 0 and must run after the other even slices as in the
serial loop of MCRotationsMove (mc_piqmc.cc:490-507)."""
import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W
from _common import golden, golden_cases

pytestmark = pytest.mark.gpu


def _state(s):
    c, a, co, p = s.get_state()
    return c, a, co, p


def _pass_pair(w, mixed, npass=2, seed=777):
    out = []
    for fused in (1, 0):
        s = G.Sampler(w, mixed=mixed)
        s.set_option(G.OPT_FUSED, fused)
        s.reset_counters()
        s.run_passes(npass, seed=seed)
        s.synchronize()
        out.append((_state(s), s.counters()))
        s.close()
    return out


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("name", golden_cases())
def test_fused_schedule_equals_phase_launches(name, mixed):
    w, d, _ = golden(name)
    if any(w.nslices % (1 << t["levels"]) for t in w.types):
        pytest.skip("production schedule needs P divisible by 2^levels")
    (sa, ca), (sb, cb) = _pass_pair(w, mixed)
    for x, y in zip(sa, sb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(ca[0], cb[0])
    np.testing.assert_array_equal(ca[1], cb[1])


@pytest.mark.parametrize("q", [2, 4])
def test_persistent_sweeps_with_few_slices(q):
    """Q = 2 (one CTA, no waits; both links join the same two slices) and
    Q = 4 (two CTAs waiting on each other)."""
    w = W.config0(seed=11, nslices=32, nrotslices=q, n_he=3)
    (sa, ca), (sb, cb) = _pass_pair(w, mixed=False, npass=3)
    for x, y in zip(sa, sb):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(ca[0], cb[0])


@pytest.mark.parametrize("P,Q", [(60, 5), (48, 3)])
def test_odd_rotational_slice_count_replays_the_serial_sweep(P, Q):
    w = W.config0(seed=5, nslices=P, nrotslices=Q, n_he=4)
    s = G.Sampler(w)
    o = O.Oracle(w)
    rng = np.random.default_rng(9)
    tau = 1.0 / (w.temperature * w.nslices)
    R = P // Q
    _, _, co0, _ = o.get_state()
    erot = max(abs(o.pot_rot_energy(4, co0, t)) for t in range(0, P, 7))
    for sweep in range(4):
        ur = rng.uniform(size=3 * Q)
        rs, rd, acc = s.rotations(ur)
        _, ord_, oacc, _ = o.rotations(1, ur)
        assert rs == 0
        np.testing.assert_array_equal(acc, oacc)
        scale = np.maximum(np.abs(ord_), 1.0) * max(1.0, tau * 2 * R * erot)
        assert (np.abs(rd - ord_) <= 1e-10 * scale).all(), np.max(np.abs(rd - ord_) / scale)
    c, a, co, _ = s.get_state()
    c2, a2, co2, _ = o.get_state()
    np.testing.assert_allclose(a, a2, rtol=0, atol=1e-12)
    s.close()
