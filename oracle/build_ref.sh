#!/bin/bash
# Compile the UNTOUCHED reference sources where they lie (read-only) into
# oracle/_ref/ with gcc and the forced-include shim oracle/ref_shim.h.
# Only possible where the reference tree is mounted; outputs never leave
# oracle/_ref/ (git-ignored).  Test infrastructure: the product never runs these.
#
#   oracle/_ref/infoli_omp.x       src/openmp/infoli.c + src/utils/utils.c
#                                   (OpenMP build, trace every 100 steps)
#   oracle/_ref/infoli_omp_test.x  same with -DG_CAL_FROM_FILE
#                                   (reference make target omp_test, src/makefile:78-82)
#   oracle/_ref/stable_version.x   src/regression_test/stable_version.c
#                                   (the regression golden generator, -DG_CAL_FROM_FILE)
#   oracle/_ref/checker.x          src/regression_test/regression_checker.c
#
# FP contraction is disabled so the float results do not depend on whether the
# target has FMA; the same flag is used for the oracle restatement.
set -euo pipefail
REF=${INFOLI_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/openmp" ]; then
  echo "reference tree not present at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
CFLAGS="-O3 -ffp-contract=off -fcommon -std=gnu89 -w -include $HERE/ref_shim.h"
gcc $CFLAGS -fopenmp "$REF/src/openmp/infoli.c" "$REF/src/utils/utils.c" -lm -o "$OUT/infoli_omp.x"
gcc $CFLAGS -fopenmp -DG_CAL_FROM_FILE "$REF/src/openmp/infoli.c" "$REF/src/utils/utils.c" -lm -o "$OUT/infoli_omp_test.x"
gcc $CFLAGS -DG_CAL_FROM_FILE "$REF/src/regression_test/stable_version.c" -lm -o "$OUT/stable_version.x"
gcc -O3 -w "$REF/src/regression_test/regression_checker.c" -lm -o "$OUT/checker.x"
install -m 644 "$REF/bin/default.conf" "$OUT/default.conf"
echo "built reference binaries into $OUT"
