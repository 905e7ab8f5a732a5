#!/usr/bin/env bash
# Builds the reference's own C (read where it lies, under /root/reference) as
# a CPU oracle: oracle/_ref/libref64.so (all CTYPE/DTYPE double, the FP64
# oracle form) and oracle/_ref/libref32.so (float CTYPE/DTYPE, as shipped).
#
# Test infrastructure only. Runs in the development container, where the
# reference is mounted; the GPU machine has no reference tree, and there the
# oracle restatement (oracle/topopt_oracle.c) stands in.
#
# The reference targets nvc OpenMP offload; gcc's host fallback needs four
# mechanical, semantics-preserving patches, applied to COPIES written under
# oracle/_ref/src*/ (git-ignored build intermediates, never committed):
#   1. strip `default(none)` (gcc 13 rejects the const locals it lists);
#   2. collapse(9) -> collapse(6) at stencil_methods.c:718 (gcc rejects the
#      `break` inside a collapsed nest; it only leaves the innermost loops);
#   3. drop `nowait` on `#pragma omp target` lines (libgomp's host fallback
#      deadlocked on them with more than one thread);
#   4. FP64 flavour only: typedef double CTYPE / DTYPE (definitions.h:27,29).
# CHOLMOD and CBLAS are replaced by the stand-ins in oracle/shims/.
set -euo pipefail
REF=${REF:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF" ]; then
  echo "build_ref: no reference tree at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
SRCS="stencil_methods.c stencil_assembly.c stencil_solvers.c stencil_grid_utility.c stencil_optimization.c local_matrix.c gpu_definitions.c"
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
  objs=""
  for f in $SRCS; do
    gcc -std=gnu11 -O2 -fPIC -fopenmp -ffp-contract=off -w -I"$S" -I"$HERE/shims" -c "$S/$f" -o "$S/${f%.c}.o"
    objs="$objs $S/${f%.c}.o"
  done
  gcc -std=gnu11 -O2 -fPIC -fopenmp -ffp-contract=off -w -I"$S" -I"$HERE/shims" -c "$HERE/ref_driver.c" -o "$S/ref_driver.o"
  gcc -std=gnu11 -O2 -fPIC -fopenmp -ffp-contract=off -w -I"$HERE/shims" -c "$HERE/shims/cblas_shim.c" -o "$S/cblas_shim.o"
  gcc -std=gnu11 -O2 -fPIC -fopenmp -ffp-contract=off -w -I"$HERE/shims" -c "$HERE/shims/cholmod_shim.c" -o "$S/cholmod_shim.o"
  gcc -shared -fopenmp -o "$OUT/libref$flavour.so" $objs "$S/ref_driver.o" "$S/cblas_shim.o" "$S/cholmod_shim.o" -lm
done
echo "build_ref: built $OUT/libref32.so $OUT/libref64.so"
