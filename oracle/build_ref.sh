#!/usr/bin/env bash
# Builds the reference's own C as a CPU oracle and CPU baseline:
# oracle/_ref/libref64.so (all CTYPE/DTYPE double, the FP64 oracle form) and
# oracle/_ref/libref32.so (float CTYPE/DTYPE, as shipped).
#
# Test infrastructure only. Where the reference tree is mounted (at
# $TOPOPT_REFERENCE_DIR, by default /root/reference) the sources are read
# there and mechanically patched copies are written under oracle/_ref/src*/
# (git-ignored build intermediates, never committed). Where it is not (the GPU
# box), the copies written earlier in oracle/_ref/src*/ are compiled if they
# are present; otherwise nothing is built.
#
# The reference targets nvc OpenMP offload; gcc's host fallback needs four
# mechanical, semantics-preserving patches:
#   1. strip `default(none)` (gcc 13 rejects the const locals it lists);
#   2. collapse(9) -> collapse(6) at stencil_methods.c:718 (gcc rejects the
#      `break` inside a collapsed nest; it only leaves the innermost loops);
#   3. drop `nowait` on `#pragma omp target` lines (libgomp's host fallback
#      deadlocked on them with more than one thread);
#   4. FP64 flavour only: typedef double CTYPE / DTYPE (definitions.h:27,29).
# CHOLMOD and CBLAS are replaced by the stand-ins in oracle/shims/.
set -euo pipefail
REF=${TOPOPT_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRCS="stencil_methods.c stencil_assembly.c stencil_solvers.c stencil_grid_utility.c stencil_optimization.c local_matrix.c gpu_definitions.c"
CFLAGS="-std=gnu11 -O3 -fPIC -fopenmp -ffp-contract=off -w"
if [ -d "$REF" ]; then
  mkdir -p "$OUT"
  for flavour in 32 64; do
    S="$OUT/src$flavour"
    rm -rf "$S"
    mkdir -p "$S"
    for f in $SRCS $(cd "$REF" && ls *.h); do
      sed -e 's/default(none)//g' \
          -e 's/collapse(9)/collapse(6)/' \
          -e '/#pragma omp target/ s/\bnowait\b//' \
          "$REF/$f" > "$S/$f"
    done
    if [ "$flavour" = 64 ]; then
      sed -i -e 's/^typedef float CTYPE;/typedef double CTYPE;/' \
             -e 's/^typedef float DTYPE;/typedef double DTYPE;/' "$S/definitions.h"
      grep -q '^typedef double CTYPE;' "$S/definitions.h"
      grep -q '^typedef double DTYPE;' "$S/definitions.h"
    fi
  done
elif [ ! -f "$OUT/src64/stencil_methods.c" ]; then
  echo "build_ref: no reference tree and no patched copies; skipping" >&2
  exit 0
fi
pids=""
for flavour in 32 64; do
  S="$OUT/src$flavour"
  [ -f "$S/stencil_methods.c" ] || continue
  for f in $SRCS; do
    gcc $CFLAGS -I"$S" -I"$HERE/shims" -c "$S/$f" -o "$S/${f%.c}.o" & pids="$pids $!"
  done
  gcc $CFLAGS -I"$S" -I"$HERE/shims" -c "$HERE/ref_driver.c" -o "$S/ref_driver.o" & pids="$pids $!"
  gcc $CFLAGS -I"$HERE/shims" -c "$HERE/shims/cblas_shim.c" -o "$S/cblas_shim.o" & pids="$pids $!"
  gcc $CFLAGS -I"$HERE/shims" -c "$HERE/shims/cholmod_shim.c" -o "$S/cholmod_shim.o" & pids="$pids $!"
done
for p in $pids; do wait "$p"; done
built=""
for flavour in 32 64; do
  S="$OUT/src$flavour"
  [ -f "$S/stencil_methods.c" ] || continue
  objs=""
  for f in $SRCS; do objs="$objs $S/${f%.c}.o"; done
  gcc -shared -fopenmp -o "$OUT/libref$flavour.so" $objs "$S/ref_driver.o" "$S/cblas_shim.o" "$S/cholmod_shim.o" -lm
  built="$built $OUT/libref$flavour.so"
done
echo "build_ref: built$built"
