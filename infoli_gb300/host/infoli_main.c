/*
 * infoli.x -- drop-in replacement for the reference's OpenMP simulator
 * executable (src/openmp/infoli.c main, :43-735) whose time-step loop runs on
 * the GPU through libinfoli_gpu.so.
 *
 * Kept from the reference:
 *   - command line getopt("hn:p:t:i:c:o:") with the same defaults (1000 cells,
 *     density 0.5, 5000 ms) and the same clamping messages (:106-167);
 *   - parameters read positionally from default.conf found beside the
 *     executable, or from -c (:113-121, src/utils/utils.c:137-160);
 *   - the built-in Bernoulli(p) topology generator with uniform CONDUCTANCE,
 *     seeded with time(NULL) (:337-375);
 *   - the hard-coded 6 uA/cm2 pulse for steps 20000..20498 (:482-485);
 *   - the output file format: header, every 100th step " %d %.2f " then
 *     "%d : %.8f " per cell (V_axon), the execution-time line rewritten in
 *     place at the end (:188-198, :383-396, :682-696, :710-732);
 *   - built with -DG_CAL_FROM_FILE (infoli_kat.x, the reference's omp_test
 *     target): g_CaL read from gcal_file.txt in the working directory, every
 *     step printed untagged, no header (:194-197, :294-296).
 * Extensions: -s <seed> fixes the generator seed (default time(NULL));
 * -K enables Kahan-compensated coupling sums.  -i is accepted like the
 * reference (which opens and then ignores the stimulus file, :169-176,
 * :430-477); -I <file> applies a per-step stimulus file in the reference's
 * format (src/utils/utils.c:70-122), one line per step, and the run lasts as
 * many steps as the file has lines (the intent of the disabled loop); the
 * Input(Iapp) column then shows cell 0's value.  -m <file> / -M <file> read
 * the connectivity from a dense conductance matrix / "send rec g" triples
 * (src/truncated/openmp-oldAPI/infoli.c:262-350) instead of the generator.
 * -R randomises the initial state (RAND_INIT, src/single_threaded/infoli.c:
 * 206-236) with the -s seed.
 * Errors are reported like the reference (printf + exit(EXIT_FAILURE)).
 */
#define _GNU_SOURCE
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <time.h>
#include <unistd.h>

#include "infoli_gpu.h"

static void print_usage(void) {
  printf("Usage for infoli simulator:\n");
  printf("/path/to/bin/infoli.x -n <integer> -p <[0,1]> -t <float>\n");
  printf("-i <filename> -c <filename> -o <filename>\n");
  printf("Argument summary:\n");
  printf("-n denotes number of neurons to be simulated. Default value: 1000.\n");
  printf("-p denotes network density in [0,1] format. Default value: 0.5 (=50%%).\n");
  printf("-t denotes simulation time in milliseconds. Default value: 5000.\n");
  printf("-i denotes a filename for input stimulus. By default, stimulus is hardcoded.\n");
  printf("-c denotes a filename for configuration file. By default, configuration is read from default.conf.\n");
  printf("-o denotes a filename for simulation output. Default value: InferiorOlive_Output.txt.\n");
  printf("-s denotes the connectivity generator seed. Default value: time(NULL).\n");
  printf("-K enables compensated (Kahan) coupling sums.\n");
  printf("-I denotes a per-step stimulus file (one line of n values per step).\n");
  printf("-m / -M denote a connectivity file: dense conductance matrix / send rec g triples.\n");
  printf("-R randomises the initial state (seeded by -s).\n");
}

struct trace_ctx {
  FILE* out;
  char* buf;
  long long cap;
  int tagged;
  int stim_start, stim_end;
  float stim_amp;
  const float* table; /* per-step stimulus (-I), row r = step r, or NULL */
  int n;
};

static void on_trace(void* user, int step, int what, const float* v, int n) {
  struct trace_ctx* t = (struct trace_ctx*)user;
  (void)what;
  if (t->tagged) {
    const float iApp = t->table ? t->table[(size_t)step * t->n]
                                : (step >= t->stim_start && step < t->stim_end) ? t->stim_amp : 0.0f;
    fprintf(t->out, " %d %.2f ", step + 1, iApp);
  }
  long long len = infoli_format_row(t->buf, t->cap, v, n, t->tagged, 0);
  if (len < 0) {
    printf("Error: trace buffer too small\n");
    exit(EXIT_FAILURE);
  }
  fwrite(t->buf, 1, (size_t)len, t->out);
}

int main(int argc, char** argv) {
  int n = 1000;
  float p = 0.5f;
  float simTime = 5000;
  int kahan = 0;
  unsigned seed = (unsigned)time(NULL);
  char* paramsFileName = (char*)malloc(PATH_MAX);
  char* outFileName = (char*)"InferiorOlive_Output.txt";
  char* inFileName = NULL;
  char* stimFileName = NULL;
  char* connFileName = NULL;
  int connTriples = 0, randInit = 0;
  char tempbuf[128];

  /* default.conf beside the executable (:113-121) */
  ssize_t l = readlink("/proc/self/exe", paramsFileName, PATH_MAX - 16);
  if (l == -1) {
    printf("Error: Couldn't read simlink to running executable.\n");
    exit(EXIT_FAILURE);
  }
  paramsFileName[l] = '\0';
  char* slash = strrchr(paramsFileName, '/');
  if (slash) slash[1] = '\0';
  else paramsFileName[0] = '\0';
  strcat(paramsFileName, "default.conf");

  int option;
  while ((option = getopt(argc, argv, "hn:p:t:i:c:o:s:KI:m:M:R")) != -1) {
    switch (option) {
      case 'h':
        print_usage();
        return 0;
      case 'n':
        n = atoi(optarg);
        if (n <= 0) {
          printf("Incorrect network size argument. Using default value of 1000.\n");
          n = 1000;
        }
        break;
      case 'p':
        p = atof(optarg);
        if (p < 0) {
          printf("Incorrect network density argument. Using default value of 0.5.\n");
          p = 0.5;
        }
        if (p == 0) printf("Warning: Simulating non-connected network (network density = 0).\n");
        if (p > 1) {
          printf("Warning: Setting network density to 1 (=100%%).\n");
          p = 1;
        }
        break;
      case 't':
        simTime = atof(optarg);
        if (simTime <= 0) {
          printf("Incorrect simulation time argument. Using default value of 5000ms.\n");
          simTime = 5000;
        }
        break;
      case 'i':
        inFileName = optarg;
        break;
      case 'c':
        paramsFileName = optarg;
        break;
      case 'o':
        outFileName = optarg;
        break;
      case 's':
        seed = (unsigned)strtoul(optarg, NULL, 10);
        break;
      case 'K':
        kahan = 1;
        break;
      case 'I':
        stimFileName = optarg;
        break;
      case 'm':
      case 'M':
        connFileName = optarg;
        connTriples = option == 'M';
        break;
      case 'R':
        randInit = 1;
        break;
      default:
        print_usage();
        exit(EXIT_FAILURE);
    }
  }
  if (inFileName) {
    FILE* f = fopen(inFileName, "r");
    if (!f) {
      printf("Error: Couldn't open %s\n", inFileName);
      exit(EXIT_FAILURE);
    }
    fclose(f); /* the reference opens and then ignores it (:169-176, :430-477) */
  }

  FILE* pOutFile = fopen(outFileName, "w+");
  if (!pOutFile) {
    printf("Error: Couldn't create %s\n", outFileName);
    exit(EXIT_FAILURE);
  }
  int print_granularity = 100;
#ifdef G_CAL_FROM_FILE
  print_granularity = 1;
#endif

  float conf[INFOLI_NCONF];
  if (infoli_read_parameters(paramsFileName, conf) != INFOLI_OK) {
    printf("%s\n", infoli_last_error());
    printf("For a proper Configuration file format, please see default.conf in bin folder.\n");
    exit(EXIT_FAILURE);
  }

  /* per-cell state (:267-292) */
  float* state = (float*)malloc(sizeof(float) * INFOLI_NSTATE * (size_t)n);
  for (int k = 0; k < INFOLI_NSTATE; k++)
    for (int c = 0; c < n; c++) state[(size_t)k * n + c] = conf[INFOLI_NPARAM + k];
#ifdef G_CAL_FROM_FILE
  if (infoli_read_gcal("gcal_file.txt", n, state + (size_t)INFOLI_S_G_CAL * n) < 0) {
    printf("%s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }
#endif

  /* connectivity (:306-375), or a connectivity file */
  int64_t* row_ptr = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
  int64_t cap = 0, ne = 0;
  int32_t* col = NULL;
  float* gedge = NULL;
  int rc;
  if (connFileName) {
    rc = connTriples ? infoli_read_conn_triples(connFileName, n, row_ptr, NULL, NULL, 0, &ne)
                     : infoli_read_conn_dense(connFileName, n, row_ptr, NULL, NULL, 0, &ne);
    if (rc == INFOLI_ERR_CAPACITY) {
      cap = ne;
      col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cap > 0 ? cap : 1));
      gedge = (float*)malloc(sizeof(float) * (size_t)(cap > 0 ? cap : 1));
      rc = connTriples ? infoli_read_conn_triples(connFileName, n, row_ptr, col, gedge, cap, &ne)
                       : infoli_read_conn_dense(connFileName, n, row_ptr, col, gedge, cap, &ne);
    }
  } else {
    cap = (int64_t)((double)n * (n - 1) * (p * 1.05 + 0.001)) + 1024;
    if (cap > (int64_t)n * (n - 1)) cap = (int64_t)n * (n - 1);
    col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cap > 0 ? cap : 1));
    rc = infoli_gen_uniform(n, p, seed, row_ptr, col, cap, &ne);
    if (rc == INFOLI_ERR_CAPACITY) {
      free(col);
      cap = ne;
      col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cap > 0 ? cap : 1));
      rc = infoli_gen_uniform(n, p, seed, row_ptr, col, cap, &ne);
    }
  }
  if (rc != INFOLI_OK) {
    printf("%s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }
  if (randInit && infoli_random_init(conf, n, seed, state, 0) != INFOLI_OK) {
    printf("Error: %s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }
  /* per-step stimulus file */
  float* stimTable = NULL;
  int64_t stimRows = 0;
  if (stimFileName) {
    rc = infoli_read_stim_file(stimFileName, n, NULL, 0, &stimRows);
    if (rc == INFOLI_OK || rc == INFOLI_ERR_CAPACITY) {
      stimTable = (float*)malloc(sizeof(float) * (size_t)(stimRows > 0 ? stimRows : 1) * (size_t)n);
      rc = infoli_read_stim_file(stimFileName, n, stimTable, stimRows, &stimRows);
    }
    if (rc != INFOLI_OK) {
      printf("%s\n", infoli_last_error());
      exit(EXIT_FAILURE);
    }
  }

#ifndef G_CAL_FROM_FILE
  sprintf(tempbuf, "Execution Time for Simulation in ms:              \n");
  fputs(tempbuf, pOutFile);
  fputs("#simSteps Input(Iapp) Output(V_axon)", pOutFile);
  for (int c = 0; c < n; c++) fprintf(pOutFile, "%d ", c);
  fputs("\n", pOutFile);
#endif

  infoli_sim_desc d;
  memset(&d, 0, sizeof d);
  d.n_cells = n;
  d.params = conf;
  d.init_state = state;
  d.row_ptr = row_ptr;
  d.col = col;
  d.g = gedge;
  d.g_uniform = conf[INFOLI_P_CONDUCTANCE];
  d.flags = kahan ? INFOLI_F_KAHAN : 0;
  d.device = 0;
  infoli_sim* sim = NULL;
  if (infoli_sim_create(&d, &sim) != INFOLI_OK) {
    printf("Error: %s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }
  free(col);
  free(gedge);
  if (stimTable && stimRows > 0 && infoli_sim_set_stimulus_table(sim, stimTable, (int)stimRows, 0) != INFOLI_OK) {
    printf("Error: %s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }

  struct trace_ctx tc;
  tc.out = pOutFile;
  tc.cap = 40LL * n + 64;
  tc.buf = (char*)malloc((size_t)tc.cap);
#ifdef G_CAL_FROM_FILE
  tc.tagged = 0;
#else
  tc.tagged = 1;
#endif
  tc.stim_start = 20000;
  tc.stim_end = 20500 - 1;
  tc.stim_amp = 6.0f;
  tc.table = stimTable;
  tc.n = n;

  const int total_simulation_steps = stimTable ? (int)stimRows : (int)(simTime / conf[INFOLI_P_DELTA]);
  struct timeval tic, toc;
  gettimeofday(&tic, NULL);
  rc = infoli_sim_run(sim, total_simulation_steps, print_granularity, INFOLI_TRACE_AXON, on_trace, &tc);
  gettimeofday(&toc, NULL);
  if (rc != INFOLI_OK) {
    printf("Error: %s\n", infoli_last_error());
    exit(EXIT_FAILURE);
  }
  fclose(pOutFile);
  chmod(outFileName, 0x01B6);

  const double ms = (toc.tv_sec * 1000.0 + ((float)(toc.tv_usec) / 1000.0)) -
                    (tic.tv_sec * 1000.0 + ((float)(tic.tv_usec) / 1000.0));
  printf("Execution Time for Simulation: %0.2f ms.\n", ms);
  pOutFile = fopen(outFileName, "rb+");
  if (pOutFile) {
#ifndef G_CAL_FROM_FILE
    sprintf(tempbuf, "Execution Time for Simulation in ms: %0.2f\n", ms);
    fputs(tempbuf, pOutFile);
#endif
    fclose(pOutFile);
  }
  infoli_sim_destroy(sim);
  free(state);
  free(row_ptr);
  free(tc.buf);
  free(stimTable);
  return 0;
}
