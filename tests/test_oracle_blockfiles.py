"""The estimators' block files against the reference's own writers.  The
reference (compiled here from its sources) computes the densities, exchange
cycles and area estimators of a path and writes them with SaveDensities1D/
2D/3D, SaveRho1D, SaveExchangeLength, SaveAreaEstimators and
SaveAreaEstim3D (mc_estim.cc:1327-1800, 2021-2085, 2596-2720); the C ABI's
writers, given the same accumulators, must write the same files (they are
byte-identical with the reference run single-threaded, as the test suite
runs it: its OpenMP density loop races on the histograms)."""
import os

import numpy as np
import pytest

import oracle as O
import pimc_gb300 as G
import workloads as W

pytestmark = [pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here (oracle/ref_build.sh)"),
              pytest.mark.skipif(not os.path.exists(G.LIBPATH), reason="library not built")]

C0S = dict(seed=11, nslices=32, nrotslices=8, n_he=4, r2d_step=0.05, c2d_step=0.04)
C1S = dict(seed=12, nslices=32, nrotslices=8, n_h2=6, grid3d=(30, 37, 19), griddens=(19, 37, 37))


def _same(pa, pb):
    """Byte-identical files, or else the same layout with every number equal
    to the 7 printed digits (a double that differs in its last bit can round
    the other way)."""
    a, b = open(pa, "rb").read(), open(pb, "rb").read()
    if a == b:
        return
    la, lb = a.decode().splitlines(), b.decode().splitlines()
    assert len(la) == len(lb), (pa, len(la), len(lb))
    for x, y in zip(la, lb):
        tx, ty = x.split(), y.split()
        assert len(tx) == len(ty) and len(x) == len(y), (pa, x, y)
        np.testing.assert_allclose(np.array(tx, float), np.array(ty, float), rtol=1.5e-6, atol=0, err_msg=pa)


def _files(d):
    return sorted(f for f in os.listdir(d))


@pytest.mark.parametrize("case", ["c0s", "c1s"])
def test_density_files(tmp_path, case):
    w = W.config0(**C0S) if case == "c0s" else W.config1(**C1S)
    r = O.Reference(w)
    _, g1, g2, g3 = r.densities()
    box = r.box_size()
    # the 3D file of the nonlinear case is 2 x 10^8 bytes: one mode there
    for mode in ((0, 1) if case == "c0s" else (0,)):
        a, b = tmp_path / ("ref%d" % mode), tmp_path / ("gb%d" % mode)
        a.mkdir()
        b.mkdir()
        r.save_densities(str(a / "blk"), 3.0, mode)
        if mode == 1:                      # the run-end call writes no 1D block files
            for f in os.listdir(a):
                if f.split(".")[-1] in ("gra", "gri", "grt") and "_sum" not in f:
                    os.remove(a / f)
        G.save_densities(w, box, str(b / "blk"), 3.0, mode, g1, g2, g3)
        assert _files(a) == _files(b) and _files(a), (_files(a), _files(b))
        for f in _files(a):
            _same(a / f, b / f)
            os.remove(a / f)                   # the 3D files are 2 x 10^8 bytes each
            os.remove(b / f)


def test_exchange_and_area_files(tmp_path):
    w = W.config0(**C0S)
    r = O.Reference(w)
    nbos = w.types[0]["numb"]
    perm = np.arange(w.natoms, dtype=np.int32)
    perm[:nbos] = np.random.default_rng(3).permutation(nbos)
    r.set_pindex(perm)
    a, b = tmp_path / "ref", tmp_path / "gb"
    a.mkdir()
    b.mkdir()
    pl = r.exchange_lengths(nbos)
    for blk in (1, 2):                      # appended lines
        r.save_exchange_length(str(a / "run"), 2.0, blk)
        G.save_exchange_length(w, str(b / "run"), 2.0, blk, 0, pl, r.pindex()[0][:nbos], 0)
    mass = r.L.ref_mass(0)
    sums = r.area_estimators()
    r.save_area_estimators(str(a / "run"), 1.0, 4)
    G.save_area_estimators(w, str(b / "run"), 1.0, 4, 0, sums, mass)
    for fr in (0, 1):
        s3 = r.area_estim3d(fr)
        r.save_area_estim3d(str(a / "run"), 1.0, 4, fr)
        G.save_area_estim3d(w, str(b / "run"), 1.0, 4, fr, 0, s3[:6], s3[6:], mass)
    assert _files(a) == _files(b) == ["run.mffs3d", "run.prl", "run.sffs3d", "run.sup"]
    for f in _files(a):
        _same(a / f, b / f)


def test_rcf_file(tmp_path):
    w = W.config0(**C0S)
    r = O.Reference(w)
    a, b = tmp_path / "ref", tmp_path / "gb"
    a.mkdir()
    b.mkdir()
    for mode in (0, 1):
        rows = r.rcf_save(str(a / "run"), 2.0, mode)
        # row 0 is what pimc_rcf returns for this path (GPU-side: test_gpu_parity)
        np.testing.assert_allclose(rows[0], O.Oracle(w).rcf(), rtol=1e-12, atol=1e-12)
        G.save_rcf(w, str(b / "run"), 2.0, mode, rows)
    assert _files(a) == _files(b) == ["run.rcf", "run_sum.rcf"]
    for f in _files(a):
        _same(a / f, b / f)


@pytest.mark.parametrize("case", ["c0s", "c1s"])
def test_energy_block(tmp_path, case):
    """One MCGetAverage sample of the fixture path and its SaveEnergy line:
    the C ABI's accumulation of the oracle's estimators (the oracle matches
    the reference's estimators to rounding) gives the same sums and file."""
    w = W.config0(**C0S) if case == "c0s" else W.config1(**C1S)
    r = O.Reference(w)
    a, b = tmp_path / "ref", tmp_path / "gb"
    a.mkdir()
    b.mkdir()
    ref = r.energy_block(a, str(a / "run"), 5)
    o = O.Oracle(w)
    nonlinear = any(t["molecule"] == 2 for t in w.types)
    rot, esq, ets = o.rot_energy(nonlinear)
    sums = G.energy_accumulate(w, [o.kin_energy(), o.pot_energy_est(), rot, esq, ets])
    np.testing.assert_allclose(sums, ref, rtol=1e-9, atol=1e-9 * np.max(np.abs(ref)))
    G.save_energy(w, str(b / "run"), 1.0, 5, sums)
    _same(a / "run.eng", b / "run.eng")
    # the run-total line (SaveSumEnergy) after the same single sample
    tot = r.sum_energy(a, 3.0)
    np.testing.assert_allclose(sums, tot, rtol=1e-9, atol=1e-9 * np.max(np.abs(tot)))
    prefix = [f for f in os.listdir(a) if f.endswith("_sum.eng")]
    assert len(prefix) == 1, os.listdir(a)
    G.save_sum_energy(w, str(b / prefix[0][:-len("_sum.eng")]), 1.0, 3.0, sums)
    _same(a / prefix[0], b / prefix[0])


def test_relative_euler_files(tmp_path):
    """SaveRho1D's run-total files: the relative Euler angles of adjacent
    rotational slices binned as GetRotE3D bins them."""
    w = W.config1(**C1S)
    r = O.Reference(w)
    a, b = tmp_path / "ref", tmp_path / "gb"
    a.mkdir()
    b.mkdir()
    t, p, c = r.rel_euler(str(a / "run"), 2.0)
    assert t.sum() == w.nrotslices and p.sum() == w.nrotslices and c.sum() == w.nrotslices
    G.save_rel_euler(w, str(b / "run"), 2.0, t, p, c)
    for f in ("run_sum.eulphi", "run_sum.eulchi", "run_sum.eulthe"):
        _same(a / f, b / f)

