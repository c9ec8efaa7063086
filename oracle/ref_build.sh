#!/bin/sh
# ref_build.sh -- TEST INFRASTRUCTURE ONLY.
# Compiles the reference's own C++ sources, unchanged, from the reference
# tree, together with oracle/ref_shim.cc (replay RNG + Fortran-leaf bindings)
# and the oracle's C leaves, into oracle/_ref/libref.so.  The reference's own
# build system is not used.  Left out on purpose:
#   mc_main.cc  -- compiled with its main() renamed (-Dmain=...): the tests
#                  call its block averages and energy writers, not its loop,
#   mc_randg.cc -- SPRNG streams, replaced by the replay generators in the shim,
#   omprng.cc   -- runif()/randomseed(), replaced by the shim.
# Usage: oracle/ref_build.sh [reference_dir]
#   (default: $PIMC_REFERENCE_DIR, else the reference tree of the build container)
set -e
REF=${1:-${PIMC_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/mc_piqmc.cc" ]; then
  echo "reference sources not found at $REF; oracle/_ref not built" >&2
  exit 2
fi
mkdir -p "$OUT"
CXXFLAGS="-O2 -fopenmp -fPIC -w -I$REF -I$HERE"
pids=""
for f in mc_piqmc mc_poten mc_utils mc_setup mc_input mc_estim mc_qworm rngstream; do
  g++ $CXXFLAGS -c "$REF/$f.cc" -o "$OUT/$f.o" &
  pids="$pids $!"
done
g++ $CXXFLAGS -Dmain=pimc_reference_main_unused -c "$REF/mc_main.cc" -o "$OUT/mc_main.o" &
pids="$pids $!"
g++ $CXXFLAGS -c "$HERE/ref_shim.cc" -o "$OUT/ref_shim.o" &
pids="$pids $!"
gcc -std=gnu11 -O2 -fopenmp -fPIC -c "$HERE/pimc_oracle.c" -o "$OUT/pimc_oracle_leaves.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
g++ -shared -fopenmp -o "$OUT/libref.so" "$OUT"/*.o -lm
echo "built $OUT/libref.so"
