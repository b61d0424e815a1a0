#!/bin/bash
# Compile the UNTOUCHED reference sources into oracle/_ref/ with gcc and the
# forced-include shim oracle/ref_shim.h.  Test infrastructure: the product
# never runs these; outputs never leave oracle/_ref/ (git-ignored).
#
# Where the reference tree is mounted (INFOLI_REFERENCE_DIR, default
# /root/reference), everything is built from the sources where they lie:
#   oracle/_ref/infoli_omp.x       src/openmp/infoli.c + src/utils/utils.c
#                                   (OpenMP build, trace every 100 steps)
#   oracle/_ref/infoli_omp_test.x  same with -DG_CAL_FROM_FILE
#                                   (reference make target omp_test, src/makefile:78-82)
#   oracle/_ref/stable_version.x   src/regression_test/stable_version.c
#                                   (the regression golden generator, -DG_CAL_FROM_FILE)
#   oracle/_ref/checker.x          src/regression_test/regression_checker.c
#   oracle/_ref/infoli_omp_perf.x  the OpenMP build again, with the compiler's
#                                   default floating-point contraction: the CPU
#                                   baseline that bench.py times
#   oracle/_ref/single_rand.x      src/single_threaded/infoli.c with its own
#                                   RAND_INIT switch at 1 (infoli.h:26, "1 for
#                                   random states"): the source is staged as is in
#                                   oracle/_ref/rand_init/ beside a copy of its
#                                   header whose only change is that line (the .c
#                                   includes "infoli.h" from its own folder); the
#                                   randomised-state golden generator
# and the three sources of the OpenMP build plus bin/default.conf are staged,
# unmodified, in oracle/_ref/src/ (git-ignored, never committed).  A working
# tree copied to a host without the reference tree (the GPU host, another
# architecture) carries that folder but no binaries; there this script builds
# infoli_omp_perf.x and infoli_omp.x from the staged copy.
#
# The parity binaries disable FP contraction so the float results do not
# depend on whether the target has FMA; the same flag is used for the oracle
# restatement.
set -euo pipefail
REF=${INFOLI_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
CFLAGS="-O3 -ffp-contract=off -fcommon -std=gnu89 -w -include $HERE/ref_shim.h"
PERF_CFLAGS="-O3 -fcommon -std=gnu89 -w -include $HERE/ref_shim.h"
if [ -d "$REF/src/openmp" ]; then
  mkdir -p "$OUT" "$SRC"
  install -m 644 "$REF/src/openmp/infoli.c" "$REF/src/openmp/infoli.h" "$REF/src/utils/utils.c" \
    "$REF/bin/default.conf" "$SRC/"
  gcc $CFLAGS -fopenmp "$REF/src/openmp/infoli.c" "$REF/src/utils/utils.c" -lm -o "$OUT/infoli_omp.x"
  gcc $CFLAGS -fopenmp -DG_CAL_FROM_FILE "$REF/src/openmp/infoli.c" "$REF/src/utils/utils.c" -lm \
    -o "$OUT/infoli_omp_test.x"
  gcc $CFLAGS -DG_CAL_FROM_FILE "$REF/src/regression_test/stable_version.c" -lm -o "$OUT/stable_version.x"
  gcc -O3 -w "$REF/src/regression_test/regression_checker.c" -lm -o "$OUT/checker.x"
  gcc $PERF_CFLAGS -fopenmp "$REF/src/openmp/infoli.c" "$REF/src/utils/utils.c" -lm -o "$OUT/infoli_omp_perf.x"
  RND="$OUT/rand_init"
  mkdir -p "$RND"
  install -m 644 "$REF/src/single_threaded/infoli.c" "$RND/infoli.c"
  sed 's/^#define RAND_INIT 0/#define RAND_INIT 1/' "$REF/src/single_threaded/infoli.h" > "$RND/infoli.h"
  grep -q '^#define RAND_INIT 1' "$RND/infoli.h"
  gcc $CFLAGS "$RND/infoli.c" -lm -o "$OUT/single_rand.x"
  install -m 644 "$REF/bin/default.conf" "$OUT/default.conf"
  echo "built reference binaries into $OUT"
elif [ -f "$SRC/infoli.c" ] && [ -f "$SRC/utils.c" ]; then
  gcc $CFLAGS -fopenmp "$SRC/infoli.c" "$SRC/utils.c" -lm -o "$OUT/infoli_omp.x"
  gcc $PERF_CFLAGS -fopenmp "$SRC/infoli.c" "$SRC/utils.c" -lm -o "$OUT/infoli_omp_perf.x"
  install -m 644 "$SRC/default.conf" "$OUT/default.conf"
  echo "built the reference OpenMP binaries into $OUT from the staged sources"
else
  echo "reference tree not present at $REF and no staged sources; nothing to build" >&2
fi
exit 0
