/*
 * Trace text formatting for the reference's output file
 * (src/openmp/infoli.c:682-696): per recorded step, "%d : %.8f " per cell
 * (1-based id, V_axon) in the normal build, "%.8f " per cell in the
 * regression build; each row ends with "\n".
 *
 * printf is the bottleneck of a GPU run at 10^4 cells, so values are
 * formatted by an exact integer routine (identical bytes to glibc's "%.8f"
 * on the float promoted to double: correctly rounded, ties to even, "-" kept
 * for negative values that round to zero) and rows are cut into blocks
 * formatted by OpenMP threads.  Values outside the fast range fall back to
 * snprintf.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/infoli_gpu.h"

static const uint64_t kPow10_8 = 100000000ull;

static inline int put_uint(char* out, uint64_t v) {
  char tmp[24];
  int k = 0;
  do {
    tmp[k++] = (char)('0' + v % 10);
    v /= 10;
  } while (v);
  for (int i = 0; i < k; i++) out[i] = tmp[k - 1 - i];
  return k;
}

/* "%.8f" of (double)v into out (at least 64 bytes); returns the length. */
static int fmt_f8(char* out, float v) {
  uint32_t bits;
  memcpy(&bits, &v, 4);
  const int neg = (int)(bits >> 31);
  const uint32_t ex = (bits >> 23) & 0xffu;
  const uint32_t man = bits & 0x7fffffu;
  if (ex == 0xffu || ex >= 127 + 31) return snprintf(out, 64, "%.8f", (double)v);
  uint64_t m;
  int e;
  if (ex == 0) {
    m = man;
    e = -149;
  } else {
    m = man | 0x800000u;
    e = (int)ex - 150;
  }
  uint64_t q;
  if (e >= 0) {
    q = (m << e) * kPow10_8;
  } else {
    const uint64_t X = m * kPow10_8; /* < 2^51 */
    const int sh = -e;
    if (sh >= 63) {
      q = 0; /* X < 2^51 < half of 2^sh: rounds to 0 */
    } else {
      q = X >> sh;
      const uint64_t r = X & ((1ull << sh) - 1);
      const uint64_t half = 1ull << (sh - 1);
      if (r > half || (r == half && (q & 1))) q++;
    }
  }
  int k = 0;
  if (neg) out[k++] = '-';
  k += put_uint(out + k, q / kPow10_8);
  out[k++] = '.';
  uint64_t f = q % kPow10_8;
  for (int i = 7; i >= 0; i--) {
    out[k + i] = (char)('0' + f % 10);
    f /= 10;
  }
  k += 8;
  out[k] = '\0';
  return k;
}

/* Exposed for tests: "%.8f" of one value. */
int infoli_format_f8(char* out, float v) { return fmt_f8(out, v); }

/* Formats one trace row (values of n cells) into buf; tagged = 1 gives
 * "%d : %.8f " with 1-based ids, 0 gives "%.8f ".  Appends "\n".  Returns the
 * number of bytes, or -1 if cap is too small (cap >= 40 * n + 2 always fits). */
int64_t infoli_format_row(char* buf, int64_t cap, const float* v, int n, int tagged, int nthreads) {
  if (n <= 0) {
    if (cap < 1) return -1;
    buf[0] = '\n';
    return 1;
  }
  const int kPer = 40; /* max bytes per formatted cell in the fast path */
  int nb = 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  if (n >= 4096) nb = nthreads;
#else
  (void)nthreads;
#endif
  if (nb > 64) nb = 64;
  int64_t offs[65];
  char* tmp = NULL;
  if (nb > 1) {
    tmp = (char*)malloc((size_t)n * kPer + 64 * (size_t)nb);
    if (!tmp) nb = 1;
  }
  if (nb == 1) {
    int64_t k = 0;
    char cell[96];
    for (int c = 0; c < n; c++) {
      int len = 0;
      if (tagged) {
        len = put_uint(cell, (uint64_t)(c + 1));
        memcpy(cell + len, " : ", 3);
        len += 3;
      }
      len += fmt_f8(cell + len, v[c]);
      cell[len++] = ' ';
      if (k + len + 1 > cap) return -1;
      memcpy(buf + k, cell, (size_t)len);
      k += len;
    }
    buf[k++] = '\n';
    return k;
  }
  const int64_t stride = (int64_t)((n + nb - 1) / nb) * kPer + 64;
  int overflow = 0;
#pragma omp parallel for num_threads(nb) schedule(static)
  for (int b = 0; b < nb; b++) {
    const int c0 = (int)((int64_t)n * b / nb), c1 = (int)((int64_t)n * (b + 1) / nb);
    char* out = tmp + (int64_t)b * stride;
    int64_t k = 0;
    char val[96];
    for (int c = c0; c < c1; c++) {
      const int len = fmt_f8(val, v[c]);
      if (len > 24) { /* outside the fast range: redo the row serially */
#pragma omp atomic write
        overflow = 1;
        break;
      }
      if (tagged) {
        k += put_uint(out + k, (uint64_t)(c + 1));
        memcpy(out + k, " : ", 3);
        k += 3;
      }
      memcpy(out + k, val, (size_t)len);
      k += len;
      out[k++] = ' ';
    }
    offs[b + 1] = k;
  }
  if (overflow) {
    free(tmp);
    return infoli_format_row(buf, cap, v, n, tagged, 1);
  }
  int64_t total = 0;
  for (int b = 0; b < nb; b++) total += offs[b + 1];
  if (total + 1 > cap) {
    free(tmp);
    return -1;
  }
  int64_t k = 0;
  for (int b = 0; b < nb; b++) {
    memcpy(buf + k, tmp + (int64_t)b * stride, (size_t)offs[b + 1]);
    k += offs[b + 1];
  }
  buf[k++] = '\n';
  free(tmp);
  return k;
}
