"""The reference-name shim binds to the reference's own program (CPU, no GPU
calls): oracle/shim_link.sh links every reference object, mc_piqmc.cc with
its four move functions renamed, with moribs-pimc_gb300/shim/pimc_gpu_shim.cc
compiled against the reference's headers; the shared object is linked with
--no-undefined and its move functions are the shim's."""
import os
import subprocess

import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here (oracle/ref_build.sh)")
def test_shim_links_into_the_reference_program():
    r = subprocess.run(["sh", os.path.join(REPO, "oracle", "shim_link.sh")], capture_output=True, text=True)
    if r.returncode == 2:
        pytest.skip("reference sources absent")
    assert r.returncode == 0, r.stderr[-2000:]
    lib = os.path.join(REPO, "oracle", "_ref", "libref_gpu.so")
    syms = subprocess.run(["nm", "-C", "--defined-only", lib], capture_output=True, text=True).stdout
    for name in ("MCBisectionMove(int, int)", "MCMolecularMove(int)", "MCRotationsMove(int)", "MCRotations3D(int)"):
        defs = [l for l in syms.splitlines() if l.endswith(" " + name)]
        assert len(defs) == 1 and " T " in defs[0], (name, defs)
        # the reference's own definition is still there, under its *_cpu name
        assert any(l.endswith(" " + name.replace("(", "_cpu(", 1)) for l in syms.splitlines()), name
    assert "PIMCPass(int, int)" in syms and "GpuShimInit(pimc_tables const*, int)" in syms
    undef = subprocess.run(["nm", "-C", "--undefined-only", lib], capture_output=True, text=True).stdout
    assert "pimc_bisection_move" in undef and "pimc_set_state" in undef
    assert os.path.exists(os.path.join(REPO, "oracle", "_ref", "pimc_gpu"))
