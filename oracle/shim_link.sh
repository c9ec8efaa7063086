#!/bin/sh
# shim_link.sh -- TEST INFRASTRUCTURE ONLY.
# Links the reference's own objects (built by ref_build.sh from the reference
# tree) with the GB300 shim in place of the move functions of mc_piqmc.cc,
# to show that the shim's definitions bind to the reference's program:
#   oracle/_ref/libref_gpu.so  every reference object, mc_piqmc.cc recompiled
#                              with MCMolecularMove / MCBisectionMove /
#                              MCRotationsMove / MCRotations3D renamed to *_cpu,
#                              moribs-pimc_gb300/shim/pimc_gpu_shim.cc (compiled
#                              with the reference's headers), the shim core and
#                              libpimc_gb300.so; linked with --no-undefined
#   oracle/_ref/pimc_gpu       the reference's own main() (mc_main.cc, pass loop
#                              PIMCPass included) on the same objects
# Usage: oracle/shim_link.sh [reference_dir]
#   (default: $PIMC_REFERENCE_DIR, else the reference tree of the build container)
set -e
REF=${1:-${PIMC_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
REPO=$(dirname "$HERE")
OUT="$HERE/_ref"
PKG="$REPO/moribs-pimc_gb300"
if [ ! -f "$REF/mc_piqmc.cc" ] || [ ! -f "$OUT/libref.so" ]; then
  echo "reference sources or oracle/_ref not found; run oracle/ref_build.sh first" >&2
  exit 2
fi
CXXFLAGS="-O2 -fopenmp -fPIC -w -I$REF -I$HERE -I$PKG/shim"
RENAME="-DMCMolecularMove=MCMolecularMove_cpu -DMCBisectionMove=MCBisectionMove_cpu"
RENAME="$RENAME -DMCRotationsMove=MCRotationsMove_cpu -DMCRotations3D=MCRotations3D_cpu"
mkdir -p "$OUT/gpu"
g++ $CXXFLAGS $RENAME -c "$REF/mc_piqmc.cc" -o "$OUT/gpu/mc_piqmc_cpu.o"
g++ $CXXFLAGS -c "$PKG/shim/pimc_gpu_shim.cc" -o "$OUT/gpu/pimc_gpu_shim.o"
g++ $CXXFLAGS -c "$PKG/shim/pimc_shim_core.cc" -o "$OUT/gpu/pimc_shim_core.o"
OBJS=""
for f in mc_poten mc_utils mc_setup mc_input mc_estim mc_qworm rngstream ref_shim pimc_oracle_leaves; do
  OBJS="$OBJS $OUT/$f.o"
done
g++ -shared -fopenmp -o "$OUT/libref_gpu.so" $OBJS "$OUT/mc_main.o" "$OUT/gpu/mc_piqmc_cpu.o" \
    "$OUT/gpu/pimc_gpu_shim.o" "$OUT/gpu/pimc_shim_core.o" -L"$PKG" -lpimc_gb300 -Wl,--no-undefined -lm
g++ $CXXFLAGS -c "$REF/mc_main.cc" -o "$OUT/gpu/mc_main_prog.o"
g++ -fopenmp -o "$OUT/pimc_gpu" $OBJS "$OUT/gpu/mc_main_prog.o" "$OUT/gpu/mc_piqmc_cpu.o" \
    "$OUT/gpu/pimc_gpu_shim.o" "$OUT/gpu/pimc_shim_core.o" -L"$PKG" -lpimc_gb300 -Wl,-rpath,"$PKG" -lm
echo "linked $OUT/libref_gpu.so and $OUT/pimc_gpu"
