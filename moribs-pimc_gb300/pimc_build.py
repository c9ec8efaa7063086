"""Build recipe of the GB300 library: nvcc for sm_103a only, in-tree.

    python moribs-pimc_gb300/pimc_build.py   -> moribs-pimc_gb300/libpimc_gb300.so

The translation units of csrc/ (SOURCES) compiled in parallel, then linked
with the CUDA runtime.  No cmake, no torch extension machinery."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libpimc_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr"]
SOURCES = ["pimc_kernels.cu", "pimc_batch.cu", "pimc_capi.cu", "pimc_tables.cu", "pimc_worm.cu", "pimc_mlp.cu", "pimc_da.cu", "pimc_io.cu",
           "pimc_stats.cu"]


def nvcc():
    for p in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        c = os.path.join(p, "bin", "nvcc")
        if p and os.path.exists(c):
            return c
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", f)
                                                                 for f in ("pimc_gb300.h", "pimc_types.h")]
    if _newer(OUT, deps + [os.path.abspath(__file__)]) and not extra:
        build_shim(verbose)
        return OUT
    objs = []

    def comp(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(comp, SOURCES))
    # --no-undefined: a missing definition fails the build, not the first load
    cmd = [nvcc(), *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", OUT, *objs, "-lcudart"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    build_shim(verbose)
    return OUT


SHIM_OUT = os.path.join(HERE, "libpimc_shim.so")


def build_shim(verbose=False):
    """The look-ahead core of the reference-name shim (shim/pimc_shim_core.cc)
    as libpimc_shim.so, linked against libpimc_gb300.so beside it.  The
    reference-facing part (shim/pimc_gpu_shim.cc) is compiled into the
    reference's own program, with the reference's headers."""
    src = os.path.join(HERE, "shim", "pimc_shim_core.cc")
    if _newer(SHIM_OUT, [src, os.path.join(HERE, "shim", "pimc_shim_core.h"), OUT]):
        return SHIM_OUT
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-o", SHIM_OUT, "-L" + HERE, "-lpimc_gb300",
           "-Wl,-rpath,$ORIGIN", "-Wl,--no-undefined"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return SHIM_OUT


if __name__ == "__main__":
    print(build(verbose=True, extra=tuple(sys.argv[1:])))
