/*
 * Forced-include shim used ONLY to compile the untouched reference sources
 * (src/openmp/infoli.c, src/utils/utils.c, src/regression_test/*.c) with gcc
 * into oracle/_ref/.  The reference targets icc; gcc needs these extras:
 *   - <mm_malloc.h> for _mm_malloc (x86 gcc ships it; other targets get a
 *     posix_memalign fallback below),
 *   - <sys/stat.h> for chmod, <time.h> for time,
 *   - a no-op __assume_aligned (an icc builtin),
 *   - a fixed RNG seed: the reference seeds srand(time(NULL))
 *     (src/openmp/infoli.c:337,399); time() is pinned to INFOLI_REF_SEED so
 *     the generated topology is reproducible.
 * This header is test infrastructure; nothing in the product includes it.
 */
#ifndef INFOLI_REF_SHIM_H
#define INFOLI_REF_SHIM_H
#include <stdlib.h>
#include <time.h>
#include <sys/stat.h>
#if defined(__x86_64__) || defined(__i386__)
#include <mm_malloc.h>
#else
static inline void *_mm_malloc(size_t sz, size_t al) {
    void *p = 0;
    if (posix_memalign(&p, al < sizeof(void *) ? sizeof(void *) : al, sz ? sz : 1)) return 0;
    return p;
}
static inline void _mm_free(void *p) { free(p); }
#endif
#define __assume_aligned(p, n) ((void)0)
#ifndef INFOLI_REF_SEED
#define INFOLI_REF_SEED 1
#endif
#define time(x) ((time_t)(INFOLI_REF_SEED))
#endif
