"""Restart files and configurations.  The production uniforms are keyed by
(seed, pass, phase, move), so a run restarted from a checkpoint with the
same seed repeats the uninterrupted run bit for bit; the xyz file keeps the
coordinates and unit vectors of IOxyz's format."""
import numpy as np
import pytest

import pimc_gb300 as G
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mixed", [False, True])
def test_restart_repeats_the_uninterrupted_run(tmp_path, mixed):
    w = W.config0(seed=3, nslices=64, nrotslices=16, n_he=4)
    a = G.Sampler(w, mixed=mixed)
    a.run_passes(2, seed=55)
    ck = tmp_path / "run.ckpt"
    a.save_checkpoint(ck)
    a.run_passes(3, seed=55)
    ref = a.get_state()
    ref_cnt = a.counters()
    b = G.Sampler(w, mixed=mixed)
    b.load_checkpoint(ck)
    b.run_passes(3, seed=55)
    got = b.get_state()
    for x, y in zip(ref, got):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(ref_cnt, b.counters()):
        np.testing.assert_array_equal(x, y)
    a.close(); b.close()


def test_checkpoint_of_another_system_is_refused(tmp_path):
    a = G.Sampler(W.config0(seed=3, nslices=64, nrotslices=16, n_he=4))
    a.save_checkpoint(tmp_path / "a.ckpt")
    b = G.Sampler(W.config0(seed=3, nslices=64, nrotslices=16, n_he=5))
    with pytest.raises(G.PimcError):
        b.load_checkpoint(tmp_path / "a.ckpt")
    a.close(); b.close()


def test_xyz_round_trip(tmp_path):
    w = W.config0(seed=4, nslices=64, nrotslices=16, n_he=3)
    a = G.Sampler(w)
    a.run_passes(1, seed=9)
    a.write_xyz(tmp_path / "c.xyz", ["He", "CO2"])
    lines = (tmp_path / "c.xyz").read_text().splitlines()
    assert int(lines[0]) == w.natoms * w.nslices and lines[2].split()[0] == "He1"
    c, an, co, p = a.get_state()
    b = G.Sampler(w)
    b.read_xyz(tmp_path / "c.xyz")
    c2, an2, co2, _ = b.get_state()
    # the file keeps IOxyz's 7 significant digits
    np.testing.assert_allclose(c2, c, rtol=1e-6, atol=1e-6)
    rot = slice((w.natoms - 1) * w.nslices, (w.natoms - 1) * w.nslices + w.nrotslices)
    np.testing.assert_allclose(co2[:, rot], co[:, rot], rtol=0, atol=2e-6)
    a.close(); b.close()


@pytest.mark.parametrize("name", ["c0s", "c1s", "c3s"])
def test_xyz_equals_the_reference_file(name, tmp_path):
    """pimc_write_xyz of a fixture's final path equals, byte for byte, the
    file the reference's IOxyz (mc_input.cc:690-794) wrote for the same path
    (fixture xyz_text; labels are the MCAtom type names)."""
    from _common import golden
    w, d, _ = golden(name)
    s = G.Sampler(w)
    s.set_state(d["coords1"], d["angles1"], w.pindex)
    s.write_xyz(tmp_path / "f.xyz", [t["name"] for t in w.types])
    got = (tmp_path / "f.xyz").read_text()
    want = str(d["xyz_text"])
    assert got == want, next((i, a, b) for i, (a, b) in enumerate(zip(got.splitlines(), want.splitlines()))
                             if a != b)
    s.close()
