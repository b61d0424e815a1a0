/*
 * Host-side pieces of the C ABI that need no GPU: error reporting, the
 * default.conf and g_CaL readers and the reference's topology generator.
 * Compiled with gcc into libinfoli_gpu.so next to the CUDA parts.
 */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/infoli_gpu.h"
#include "infoli_internal.h"

static __thread char g_errbuf[512];

const char* infoli_last_error(void) { return g_errbuf; }

int infoli__fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof g_errbuf, fmt, ap);
  va_end(ap);
  return code;
}

void infoli__clear_error(void) { g_errbuf[0] = '\0'; }

int infoli_version(void) { return INFOLI_ABI_VERSION; }

/* src/utils/utils.c:137-160: fscanf("%s = %f\n") for 42 lines; the reference
 * exits on the first line that does not match, here the status reports it. */
int infoli_read_parameters(const char* path, float values[INFOLI_NCONF]) {
  char name[128];
  infoli__clear_error();
  if (!path || !values) return infoli__fail(INFOLI_ERR_ARG, "read_parameters: null argument");
  FILE* fd = fopen(path, "r");
  if (!fd) return infoli__fail(INFOLI_ERR_FILE, "Couldn't open %s", path);
  for (int i = 0; i < INFOLI_NCONF; i++) {
    if (fscanf(fd, "%127s = %f\n", name, &values[i]) != 2) {
      fclose(fd);
      return infoli__fail(INFOLI_ERR_CONFIG,
                          "Configuration Error: Improper Parameter %s in file %s, line %d.", name, path,
                          i + 1);
    }
  }
  fclose(fd);
  return INFOLI_OK;
}

/* src/utils/utils.c:124-135: fscanf("%f ") n times; values past the end of
 * the file are left untouched. */
int infoli_read_gcal(const char* path, int n, float* g_cal) {
  infoli__clear_error();
  if (!path || (n > 0 && !g_cal) || n < 0) return infoli__fail(INFOLI_ERR_ARG, "read_gcal: bad argument");
  FILE* fd = fopen(path, "r");
  if (!fd) return infoli__fail(INFOLI_ERR_FILE, "Couldn't open %s", path);
  int got = 0;
  for (int i = 0; i < n; i++) {
    float v;
    if (fscanf(fd, "%f ", &v) != 1) break;
    g_cal[i] = v;
    got++;
  }
  fclose(fd);
  return got;
}

/* src/openmp/infoli.c:337-375.  The draw sequence is the C library's rand()
 * after srand(seed), consumed receiver-major, sender ascending, self skipped. */
int infoli_gen_uniform(int n, float p, unsigned seed, int64_t* row_ptr, int32_t* col, int64_t cap,
                       int64_t* n_edges) {
  infoli__clear_error();
  if (n <= 0 || !row_ptr || cap < 0 || (cap > 0 && !col))
    return infoli__fail(INFOLI_ERR_ARG, "gen_uniform: bad argument");
  int64_t e = 0;
  srand(seed);
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) {
    for (int s = 0; s < n; s++) {
      if (s == r) continue;
      float rndm = ((float)rand()) / ((float)RAND_MAX);
      if (rndm <= p) {
        if (e < cap) col[e] = s;
        e++;
      }
    }
    row_ptr[r + 1] = e;
  }
  if (n_edges) *n_edges = e;
  if (e > cap) return infoli__fail(INFOLI_ERR_CAPACITY, "gen_uniform: %lld edges exceed capacity %lld",
                                   (long long)e, (long long)cap);
  return INFOLI_OK;
}

/* ---- synthetic topologies beyond the reference's generator ----------------
 * Random numbers: splitmix64 (S. Vigna's published 64-bit mixer over a
 * Weyl sequence), integer-only so every platform draws the same stream;
 * uniform floats use the top 24 bits (exact in FP32). */
static inline uint64_t sm64_next(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline float sm64_unit(uint64_t* s) { return (float)(sm64_next(s) >> 40) * (1.0f / 16777216.0f); }

/* Cells on a rows x cols grid (id = row * cols + col).  For each receiver,
 * every other cell within Euclidean distance `radius` (in cells) is a sender
 * with probability exp(-d^2 / (2 sigma^2)); candidates are visited in
 * ascending sender id and each takes one draw.  The acceptance threshold is
 * tabulated per integer d^2 as a 24-bit fixed-point number, so the draw
 * comparison is exact integer arithmetic. */
int infoli_gen_grid_gaussian(int rows, int cols, float sigma, float radius, uint64_t seed, int64_t* row_ptr,
                             int32_t* col, int64_t cap, int64_t* n_edges) {
  infoli__clear_error();
  if (rows <= 0 || cols <= 0 || sigma <= 0 || radius < 0 || !row_ptr || cap < 0 || (cap > 0 && !col))
    return infoli__fail(INFOLI_ERR_ARG, "gen_grid_gaussian: bad argument");
  const int R = (int)radius;
  const int r2max = (int)(radius * radius);
  uint32_t* thr = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(r2max + 1));
  if (!thr) return infoli__fail(INFOLI_ERR_NOMEM, "gen_grid_gaussian: out of memory");
  for (int d2 = 0; d2 <= r2max; d2++) {
    double pr = exp(-(double)d2 / (2.0 * (double)sigma * (double)sigma));
    thr[d2] = (uint32_t)(pr * 16777216.0);
  }
  const int n = rows * cols;
  uint64_t st = seed;
  int64_t e = 0;
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) {
    const int ry = r / cols, rx = r % cols;
    const int y0 = ry - R < 0 ? 0 : ry - R, y1 = ry + R >= rows ? rows - 1 : ry + R;
    const int x0 = rx - R < 0 ? 0 : rx - R, x1 = rx + R >= cols ? cols - 1 : rx + R;
    for (int y = y0; y <= y1; y++) {
      for (int x = x0; x <= x1; x++) {
        const int dy = y - ry, dx = x - rx, d2 = dy * dy + dx * dx;
        if (d2 == 0 || d2 > r2max) continue;
        const uint32_t u = (uint32_t)(sm64_next(&st) >> 40);
        if (u < thr[d2]) {
          if (e < cap) col[e] = y * cols + x;
          e++;
        }
      }
    }
    row_ptr[r + 1] = e;
  }
  free(thr);
  if (n_edges) *n_edges = e;
  if (e > cap) return infoli__fail(INFOLI_ERR_CAPACITY, "gen_grid_gaussian: %lld edges exceed capacity %lld",
                                   (long long)e, (long long)cap);
  return INFOLI_OK;
}

/* Each receiver draws k distinct senders uniformly from the other n-1 cells
 * (rejection of self and repeats), listed in ascending id; when g is not
 * NULL each edge also gets a conductance uniform in [g_lo, g_hi).  Needs
 * cap >= n * k. */
int infoli_gen_fixed_degree(int n, int k, float g_lo, float g_hi, uint64_t seed, int64_t* row_ptr, int32_t* col,
                            float* g, int64_t cap) {
  infoli__clear_error();
  if (n <= 1 || k < 0 || k > n - 1 || !row_ptr || (int64_t)n * k > cap || (k > 0 && !col))
    return infoli__fail(INFOLI_ERR_ARG, "gen_fixed_degree: bad argument");
  uint8_t* mark = (uint8_t*)calloc((size_t)n, 1);
  int32_t* pick = (int32_t*)malloc(sizeof(int32_t) * (size_t)(k > 0 ? k : 1));
  if (!mark || !pick) {
    free(mark);
    free(pick);
    return infoli__fail(INFOLI_ERR_NOMEM, "gen_fixed_degree: out of memory");
  }
  uint64_t st = seed;
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) {
    int got = 0;
    while (got < k) {
      const int s = (int)((sm64_next(&st) >> 32) % (uint64_t)n);
      if (s == r || mark[s]) continue;
      mark[s] = 1;
      pick[got++] = s;
    }
    /* ascending ids: counting over the marks of this row */
    int64_t base = (int64_t)r * k;
    int w = 0;
    for (int i = 0; i < got; i++) mark[pick[i]] = 2;
    /* insertion by scanning the picked ids in sorted order */
    for (int i = 1; i < got; i++) {
      int32_t v = pick[i];
      int j = i - 1;
      while (j >= 0 && pick[j] > v) {
        pick[j + 1] = pick[j];
        j--;
      }
      pick[j + 1] = v;
    }
    for (int i = 0; i < got; i++) {
      col[base + w] = pick[i];
      if (g) g[base + w] = g_lo + (g_hi - g_lo) * sm64_unit(&st);
      w++;
      mark[pick[i]] = 0;
    }
    row_ptr[r + 1] = base + w;
  }
  free(mark);
  free(pick);
  return INFOLI_OK;
}

int infoli_bitmask_to_csr(int n, const uint32_t* bits, int64_t* row_ptr, int32_t* col, int64_t cap,
                          int64_t* n_edges) {
  infoli__clear_error();
  if (n <= 0 || !bits || !row_ptr || cap < 0 || (cap > 0 && !col))
    return infoli__fail(INFOLI_ERR_ARG, "bitmask_to_csr: bad argument");
  const int64_t words = (n + 31) / 32;
  int64_t e = 0;
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) {
    const uint32_t* row = bits + (int64_t)r * words;
    for (int64_t w = 0; w < words; w++) {
      uint32_t x = row[w];
      while (x) {
        int b = __builtin_ctz(x);
        x &= x - 1;
        int64_t s = w * 32 + b;
        if (s >= n) break;
        if (e < cap) col[e] = (int32_t)s;
        e++;
      }
    }
    row_ptr[r + 1] = e;
  }
  if (n_edges) *n_edges = e;
  if (e > cap) return infoli__fail(INFOLI_ERR_CAPACITY, "bitmask_to_csr: %lld edges exceed capacity %lld",
                                   (long long)e, (long long)cap);
  return INFOLI_OK;
}

/* Receiver r draws from its own splitmix64 stream, one draw per sender in
 * ascending order (self skipped), so rows are independent of each other and
 * of the thread that makes them. */
int infoli_gen_bitmask(int n, float p, uint64_t seed, uint32_t* bits) {
  infoli__clear_error();
  if (n <= 0 || !bits || !(p >= 0.0f)) return infoli__fail(INFOLI_ERR_ARG, "gen_bitmask: bad argument");
  const int64_t words = (n + 31) / 32;
  const double pt = (double)p * 16777216.0;
  const uint32_t thr = pt >= 16777216.0 ? 16777216u : (uint32_t)pt;
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < n; r++) {
    uint64_t st = seed + (uint64_t)(r + 1) * 0x632BE59BD9B4E019ull;
    uint32_t* row = bits + (int64_t)r * words;
    for (int64_t w = 0; w < words; w++) row[w] = 0;
    for (int s = 0; s < n; s++) {
      if (s == r) continue;
      const uint32_t u = (uint32_t)(sm64_next(&st) >> 40);
      if (u < thr) row[s >> 5] |= 1u << (s & 31);
    }
  }
  return INFOLI_OK;
}

/* CSR of infoli_gen_bitmask's matrix without building the bitmask: the same
 * per-receiver streams, one pass to count each row and one to fill it, both
 * parallel over receivers. */
int infoli_gen_bitmask_csr(int n, float p, uint64_t seed, int64_t* row_ptr, int32_t* col, int64_t cap,
                           int64_t* n_edges) {
  infoli__clear_error();
  if (n <= 0 || !row_ptr || !(p >= 0.0f) || cap < 0 || (cap > 0 && !col))
    return infoli__fail(INFOLI_ERR_ARG, "gen_bitmask_csr: bad argument");
  const double pt = (double)p * 16777216.0;
  const uint32_t thr = pt >= 16777216.0 ? 16777216u : (uint32_t)pt;
  row_ptr[0] = 0;
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < n; r++) {
    uint64_t st = seed + (uint64_t)(r + 1) * 0x632BE59BD9B4E019ull;
    int64_t k = 0;
    for (int s = 0; s < n; s++) {
      if (s == r) continue;
      if ((uint32_t)(sm64_next(&st) >> 40) < thr) k++;
    }
    row_ptr[r + 1] = k;
  }
  for (int r = 0; r < n; r++) row_ptr[r + 1] += row_ptr[r];
  const int64_t e = row_ptr[n];
  if (n_edges) *n_edges = e;
  if (e > cap) return infoli__fail(INFOLI_ERR_CAPACITY, "gen_bitmask_csr: %lld edges exceed capacity %lld",
                                   (long long)e, (long long)cap);
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < n; r++) {
    uint64_t st = seed + (uint64_t)(r + 1) * 0x632BE59BD9B4E019ull;
    int64_t k = row_ptr[r];
    for (int s = 0; s < n; s++) {
      if (s == r) continue;
      if ((uint32_t)(sm64_next(&st) >> 40) < thr) col[k++] = s;
    }
  }
  return INFOLI_OK;
}

/* ---- connectivity and stimulus files ------------------------------------ */

#define INFOLI_MIN_COND 0.0000001f /* conductances below this are no connection */

/* src/truncated/openmp-oldAPI/infoli.c:262-311: n lines of n conductances;
 * value j of line i is the conductance from sender i to receiver j.  Two
 * passes like the reference (count, then fill), so receivers list their
 * senders in ascending order.  A short file is an error here (the reference
 * would reuse the last value read). */
int infoli_read_conn_dense(const char* path, int n, int64_t* row_ptr, int32_t* col, float* g, int64_t cap,
                           int64_t* n_edges) {
  infoli__clear_error();
  if (!path || n <= 0 || !row_ptr || cap < 0 || (cap > 0 && (!col || !g)))
    return infoli__fail(INFOLI_ERR_ARG, "read_conn_dense: bad argument");
  FILE* f = fopen(path, "r");
  if (!f) return infoli__fail(INFOLI_ERR_FILE, "Error: Couldn't open %s", path);
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cnt) {
    fclose(f);
    return infoli__fail(INFOLI_ERR_NOMEM, "read_conn_dense: out of memory");
  }
  float v;
  for (int s = 0; s < n; s++)
    for (int r = 0; r < n; r++) {
      if (fscanf(f, "%f ", &v) != 1) {
        free(cnt);
        fclose(f);
        return infoli__fail(INFOLI_ERR_CONFIG, "Error: %s holds fewer than %d x %d conductances (line %d)", path,
                            n, n, s + 1);
      }
      if (!(v < INFOLI_MIN_COND)) cnt[r + 1]++;
    }
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) row_ptr[r + 1] = row_ptr[r] + cnt[r + 1];
  const int64_t e = row_ptr[n];
  if (n_edges) *n_edges = e;
  if (e > cap) {
    free(cnt);
    fclose(f);
    return infoli__fail(INFOLI_ERR_CAPACITY, "read_conn_dense: %lld edges exceed capacity %lld", (long long)e,
                        (long long)cap);
  }
  for (int r = 0; r < n; r++) cnt[r] = row_ptr[r];
  rewind(f);
  for (int s = 0; s < n; s++)
    for (int r = 0; r < n; r++) {
      if (fscanf(f, "%f ", &v) != 1) break; /* cannot happen: the first pass read them */
      if (!(v < INFOLI_MIN_COND)) {
        col[cnt[r]] = s;
        g[cnt[r]] = v;
        cnt[r]++;
      }
    }
  free(cnt);
  fclose(f);
  return INFOLI_OK;
}

/* src/truncated/openmp-oldAPI/infoli.c:312-350: lines "send rec g"; receivers
 * keep their senders in file order.  Ids outside [0, n) are an error (the
 * reference would index out of bounds). */
int infoli_read_conn_triples(const char* path, int n, int64_t* row_ptr, int32_t* col, float* g, int64_t cap,
                             int64_t* n_edges) {
  infoli__clear_error();
  if (!path || n <= 0 || !row_ptr || cap < 0 || (cap > 0 && (!col || !g)))
    return infoli__fail(INFOLI_ERR_ARG, "read_conn_triples: bad argument");
  FILE* f = fopen(path, "r");
  if (!f) return infoli__fail(INFOLI_ERR_FILE, "Error: Couldn't open %s", path);
  int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  if (!cnt) {
    fclose(f);
    return infoli__fail(INFOLI_ERR_NOMEM, "read_conn_triples: out of memory");
  }
  int snd, rec, rc;
  float v;
  long long line = 0;
  while ((rc = fscanf(f, "%d %d %f\n", &snd, &rec, &v)) != EOF) {
    line++;
    if (rc != 3 || snd < 0 || snd >= n || rec < 0 || rec >= n) {
      free(cnt);
      fclose(f);
      return infoli__fail(INFOLI_ERR_CONFIG, "Error: %s line %lld is not \"send rec g\" with ids below %d", path,
                          line, n);
    }
    if (!(v < INFOLI_MIN_COND)) cnt[rec + 1]++;
  }
  row_ptr[0] = 0;
  for (int r = 0; r < n; r++) row_ptr[r + 1] = row_ptr[r] + cnt[r + 1];
  const int64_t e = row_ptr[n];
  if (n_edges) *n_edges = e;
  if (e > cap) {
    free(cnt);
    fclose(f);
    return infoli__fail(INFOLI_ERR_CAPACITY, "read_conn_triples: %lld edges exceed capacity %lld", (long long)e,
                        (long long)cap);
  }
  for (int r = 0; r < n; r++) cnt[r] = row_ptr[r];
  rewind(f);
  while (fscanf(f, "%d %d %f\n", &snd, &rec, &v) == 3) {
    if (!(v < INFOLI_MIN_COND)) {
      col[cnt[rec]] = snd;
      g[cnt[rec]] = v;
      cnt[rec]++;
    }
  }
  free(cnt);
  fclose(f);
  return INFOLI_OK;
}

/* src/utils/utils.c:70-122 (ReadFileLine): one line per step, values
 * separated by single spaces; the first n of a line are the cells' iApp
 * (atof, stored as float).  A line with fewer than n space-separated fields
 * is an error, counted like the reference (a trailing space before the
 * newline counts as a field).  Lines have no length limit here. */
int infoli_read_stim_file(const char* path, int n, float* table, int64_t max_rows, int64_t* rows) {
  infoli__clear_error();
  if (!path || n <= 0 || max_rows < 0 || (max_rows > 0 && !table) || !rows)
    return infoli__fail(INFOLI_ERR_ARG, "read_stim_file: bad argument");
  FILE* f = fopen(path, "r");
  if (!f) return infoli__fail(INFOLI_ERR_FILE, "Error: Couldn't open %s", path);
  char* line = NULL;
  size_t len = 0;
  int64_t r = 0;
  while (getline(&line, &len, f) != -1) {
    int i = 0;
    char* save = NULL;
    for (char* tok = strtok_r(line, " ", &save); tok; tok = strtok_r(NULL, " ", &save), i++)
      if (i < n && r < max_rows) table[(size_t)r * n + i] = (float)atof(tok);
    if (i < n) {
      free(line);
      fclose(f);
      return infoli__fail(INFOLI_ERR_CONFIG, "Error: Input line doesn't have enough elements, only %d", i);
    }
    r++;
  }
  free(line);
  fclose(f);
  *rows = r;
  if (r > max_rows)
    return infoli__fail(INFOLI_ERR_CAPACITY, "read_stim_file: %lld lines exceed capacity %lld", (long long)r,
                        (long long)max_rows);
  return INFOLI_OK;
}
