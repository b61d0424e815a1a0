/*
 * infoli_gpu.h -- C ABI of the GB300 InfOli network-update library
 * (libinfoli_gpu.so).
 *
 * The reference simulator has no library API: its per-step network update is
 * inline in main() of src/openmp/infoli.c.  Each entry point below replaces one
 * piece of that program, cited as file:line inside the reference project.
 * Plain C types only (pointers, sizes); no CUDA or framework types appear.
 *
 * Conventions
 *   - Every call returns an int status: INFOLI_OK (0) or a negative
 *     INFOLI_ERR_* code; infoli_last_error() gives a message for the calling
 *     thread.  Nothing here calls exit() (the reference printf()s and exits).
 *   - Host arrays passed in are copied; the caller keeps ownership.
 *   - Device memory is owned by the library and released by *_destroy.
 *   - A handle is not thread-safe; distinct handles may be used from distinct
 *     threads (each has its own CUDA streams).
 *   - Per-cell state is exchanged as 19 SoA arrays of n floats each, in the
 *     order of bin/default.conf lines 24-42 (INFOLI_S_* below).
 */
#ifndef INFOLI_GPU_H
#define INFOLI_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define INFOLI_ABI_VERSION 1

/* status codes */
#define INFOLI_OK 0
#define INFOLI_ERR_ARG (-1)       /* invalid argument */
#define INFOLI_ERR_CUDA (-2)      /* CUDA runtime error / no usable GPU */
#define INFOLI_ERR_NOMEM (-3)     /* host or device allocation failed */
#define INFOLI_ERR_TIMEOUT (-4)   /* a device-side wait gave up (error recorded, kernel returned) */
#define INFOLI_ERR_FILE (-5)      /* a file could not be opened / read */
#define INFOLI_ERR_CONFIG (-6)    /* malformed configuration / input file */
#define INFOLI_ERR_CAPACITY (-7)  /* request exceeds a configured capacity (HBM budget, slots) */
#define INFOLI_ERR_STATE (-8)     /* call not valid in the handle's current state */

/* number of model constants / per-cell state arrays (bin/default.conf:1-23 / 24-42) */
#define INFOLI_NPARAM 23
#define INFOLI_NSTATE 19
#define INFOLI_NCONF 42

/* model constant indices (bin/default.conf:1-23; src/openmp/infoli.c:240-262) */
enum {
  INFOLI_P_DELTA = 0, INFOLI_P_CONDUCTANCE, INFOLI_P_C_M, INFOLI_P_G_NA_S, INFOLI_P_G_KDR_S,
  INFOLI_P_G_K_S, INFOLI_P_G_LS, INFOLI_P_G_K_CA, INFOLI_P_G_CAH, INFOLI_P_G_LD, INFOLI_P_G_H,
  INFOLI_P_G_NA_A, INFOLI_P_G_NA_R, INFOLI_P_G_K_A, INFOLI_P_G_LA, INFOLI_P_P1, INFOLI_P_P2,
  INFOLI_P_G_INT, INFOLI_P_V_NA, INFOLI_P_V_K, INFOLI_P_V_CA, INFOLI_P_V_H, INFOLI_P_V_L
};

/* state array indices (bin/default.conf:24-42; src/openmp/infoli.c:267-292) */
enum {
  INFOLI_S_V_DEND = 0, INFOLI_S_CALCIUM_R, INFOLI_S_POTASSIUM_S, INFOLI_S_HCURRENT_Q,
  INFOLI_S_CA2PLUS, INFOLI_S_I_CAH, INFOLI_S_G_CAL, INFOLI_S_V_SOMA, INFOLI_S_SODIUM_M,
  INFOLI_S_SODIUM_H, INFOLI_S_POTASSIUM_N, INFOLI_S_POTASSIUM_P, INFOLI_S_POTASSIUM_X_S,
  INFOLI_S_CALCIUM_K, INFOLI_S_CALCIUM_L, INFOLI_S_V_AXON, INFOLI_S_SODIUM_M_A,
  INFOLI_S_SODIUM_H_A, INFOLI_S_POTASSIUM_X_A
};

/* trace selection bits for infoli_sim_run */
#define INFOLI_TRACE_AXON 1 /* V_axon: what the reference prints (src/openmp/infoli.c:687) */
#define INFOLI_TRACE_SOMA 2
#define INFOLI_TRACE_DEND 4

/* flags for infoli_sim_desc.flags */
#define INFOLI_F_KAHAN 1     /* Kahan-compensated FP32 coupling sums */

/* ------------------------------------------------------------------------ */
/* library                                                                   */
/* ------------------------------------------------------------------------ */

/* Message describing the last failed call on this thread ("" if none). */
const char* infoli_last_error(void);

/* ABI version (INFOLI_ABI_VERSION) and a build description string. */
int infoli_version(void);
const char* infoli_build_info(void);

/* Number of usable CUDA devices, or a negative status. */
int infoli_device_count(void);

/* ------------------------------------------------------------------------ */
/* configuration and topology (host side)                                   */
/* ------------------------------------------------------------------------ */

/* Replaces read_parameters (src/utils/utils.c:137-160): reads the 42
 * positional "NAME = value" lines of a default.conf-style file into
 * values[42].  Names are not checked, as in the reference. */
int infoli_read_parameters(const char* path, float values[INFOLI_NCONF]);

/* Replaces read_g_CaL_from_file (src/utils/utils.c:124-135): reads up to n
 * whitespace-separated floats into g_cal; cells beyond the end of the file
 * keep their value (the reference leaves them at the default.conf value).
 * Returns the number of values read (>= 0) or a negative status. */
int infoli_read_gcal(const char* path, int n, float* g_cal);

/* Replaces the built-in topology generator (src/openmp/infoli.c:337-375):
 * srand(seed), then one rand() draw per ordered pair (receiver-major, sender
 * ascending, self skipped); an edge exists when
 * (float)rand()/(float)RAND_MAX <= p.  Output in CSR form: row_ptr[n+1] and
 * col[] (capacity cap) with ascending senders per receiver.  *n_edges gets
 * the edge count; if it exceeds cap, INFOLI_ERR_CAPACITY is returned and
 * row_ptr is still complete.  Uses the C library's rand() exactly like the
 * reference, so results are bit-identical for the same seed. */
int infoli_gen_uniform(int n, float p, unsigned seed, int64_t* row_ptr, int32_t* col, int64_t cap,
                       int64_t* n_edges);

/* Synthetic 2-D grid topology (no counterpart in the reference's CLI; its
 * nearest relatives are src/utils/utils.c:202-303 and
 * tools/connectivity/2d_gaussian/conn_generator.c:43-128): rows x cols cells,
 * id = row * cols + col; every other cell within `radius` is a sender with
 * probability exp(-d^2 / (2 sigma^2)), one splitmix64 draw per candidate in
 * ascending id.  Same output contract as infoli_gen_uniform. */
int infoli_gen_grid_gaussian(int rows, int cols, float sigma, float radius, uint64_t seed, int64_t* row_ptr,
                             int32_t* col, int64_t cap, int64_t* n_edges);

/* Synthetic sparse topology: each receiver gets k distinct uniformly drawn
 * senders (ascending ids); g (optional) gets per-edge conductances uniform in
 * [g_lo, g_hi).  cap must be >= n * k. */
int infoli_gen_fixed_degree(int n, int k, float g_lo, float g_hi, uint64_t seed, int64_t* row_ptr, int32_t* col,
                            float* g, int64_t cap);

/* Converts a dense receiver bitmask (row r = receiver, bit s of word s/32 =
 * sender s, ceil(n/32) words per row) to CSR.  Same output contract as
 * infoli_gen_uniform. */
int infoli_bitmask_to_csr(int n, const uint32_t* bits, int64_t* row_ptr, int32_t* col, int64_t cap,
                          int64_t* n_edges);

/* Dense random topology as a receiver bitmask (layout of
 * infoli_bitmask_to_csr), the bitmask form of the reference's uniform
 * generator (src/openmp/infoli.c:337-375) for the batched path: pair
 * (r, s), s != r, is an edge when a 24-bit draw is below p * 2^24.  Receiver
 * r draws from its own splitmix64 stream (state seed + (r + 1) * 0x632BE59BD9B4E019),
 * one draw per sender in ascending order, so rows are generated in parallel
 * and the result does not depend on the thread count. */
int infoli_gen_bitmask(int n, float p, uint64_t seed, uint32_t* bits);
/* The same matrix in CSR form (infoli_gen_uniform's output contract),
 * generated without the bitmask. */
int infoli_gen_bitmask_csr(int n, float p, uint64_t seed, int64_t* row_ptr, int32_t* col, int64_t cap,
                           int64_t* n_edges);

/* Connectivity files of the reference's older simulator
 * (src/truncated/openmp-oldAPI/infoli.c:262-350), read into CSR by receiver
 * with per-edge conductances (same output contract as infoli_gen_uniform,
 * plus g[cap]); conductances below 1e-7 are no connection.
 *   dense:   n lines of n values, value j of line i = conductance from
 *            sender i to receiver j (writers: tools/connectivity/percentage,
 *            3d_gaussian, 3d_synapse_count); receivers list senders ascending;
 *   triples: lines "send rec g" (tools/connectivity/3d_gaussian_compressed,
 *            3d_synapse_count); receivers list senders in file order.
 * A short dense file, a malformed line or an id outside [0, n) is
 * INFOLI_ERR_CONFIG (the reference reads past such input silently). */
int infoli_read_conn_dense(const char* path, int n, int64_t* row_ptr, int32_t* col, float* g, int64_t cap,
                           int64_t* n_edges);
int infoli_read_conn_triples(const char* path, int n, int64_t* row_ptr, int32_t* col, float* g, int64_t cap,
                             int64_t* n_edges);

/* Per-step stimulus file (-i; src/utils/utils.c:70-122 ReadFileLine): one
 * line per step, the first n space-separated values of a line are the cells'
 * iApp for that step.  Fills table[rows][n] (capacity max_rows rows; table
 * may be NULL with max_rows 0 to count lines) and sets *rows.
 * INFOLI_ERR_CAPACITY when the file has more lines than max_rows (*rows is
 * still the line count); a line with fewer than n values is
 * INFOLI_ERR_CONFIG with the reference's message. */
int infoli_read_stim_file(const char* path, int n, float* table, int64_t max_rows, int64_t* rows);

/* Randomised initial state (the reference's RAND_INIT, run by
 * src/single_threaded/infoli.c:206-236, a placeholder in
 * src/openmp/infoli.c:402-422): srand(seed), then g_CaL[c] = 0.6 +
 * 0.2 * (rand() % 100) / 100 for every cell, then every cell c draws
 * k = (rand() % ceil(100 / DELTA)) | 1 and runs on its own (no coupling
 * current, no stimulus) from its state in state[19 * n], which is overwritten
 * with the state after k - 1 steps: the reference's last isolated step lands
 * in the state buffer its simulation does not start from
 * (src/single_threaded/infoli.c:227-228, :293, :316).  Uses the C library's
 * rand() like the reference (process-wide generator state).  The isolated
 * steps run on the GPU. */
int infoli_random_init(const float* params, int n, unsigned seed, float* state, int device);

/* ------------------------------------------------------------------------ */
/* one simulation on the GPU                                                */
/* ------------------------------------------------------------------------ */

typedef struct infoli_sim infoli_sim;

typedef struct {
  int n_cells;
  const float* params;       /* [INFOLI_NPARAM] model constants */
  const float* init_state;   /* [INFOLI_NSTATE * n_cells] SoA, or NULL: broadcast init_values */
  const float* init_values;  /* [INFOLI_NSTATE] used when init_state is NULL (conf lines 24-42) */
  /* topology, CSR by receiver (the reference's cellCompParams,
   * src/openmp/infoli.h:79-83: total_amount_of_neighbours / neighId /
   * neighConductances) */
  const int64_t* row_ptr;    /* [n_cells + 1] */
  const int32_t* col;        /* [row_ptr[n]] sender ids */
  const float* g;            /* [row_ptr[n]] per-edge conductance, or NULL */
  float g_uniform;           /* conductance of every edge when g is NULL (CONDUCTANCE) */
  int flags;                 /* INFOLI_F_* */
  int device;                /* CUDA device ordinal */
  int grid;                  /* CTAs (one per SM) the simulation may use; 0 = all SMs */
} infoli_sim_desc;

/* Trace callback: called once per recorded step with the values of that step
 * (n_cells floats per selected quantity, in the order axon, soma, dend of the
 * selected bits).  step = the reference's simStep (0-based). */
typedef void (*infoli_trace_cb)(void* user, int step, int what, const float* values, int n_cells);

/* Replaces the setup half of main() (state arrays src/openmp/infoli.c:204-292,
 * connectivity :306-375): uploads parameters, state and topology and plans
 * the persistent step kernel. */
int infoli_sim_create(const infoli_sim_desc* desc, infoli_sim** out);

/* Stimulus.  Default: the reference's hard-coded pulse
 * (src/openmp/infoli.c:482-485): 6 uA/cm2 for 20000 <= step < 20499. */
int infoli_sim_set_stimulus_pulse(infoli_sim* s, int start_step, int end_step, float amp);
/* Per-cell pulses: amp[c] for onset[c] <= step < onset[c] + duration. */
int infoli_sim_set_stimulus_cells(infoli_sim* s, const float* amp, const int* onset, int duration);
/* Per-step stimulus table (the reference's stimulus file): table[r][c] is
 * cell c's iApp at step first_step + r, for rows rows; the table is copied
 * to the device.  Runs must stay inside [first_step, first_step + rows)
 * (INFOLI_ERR_ARG otherwise). */
int infoli_sim_set_stimulus_table(infoli_sim* s, const float* table, int rows, int first_step);

/* Replaces the time-step loop (src/openmp/infoli.c:478-698): advances
 * n_steps explicit-Euler steps.  When trace_every > 0, the selected
 * quantities are recorded after every step whose index is a multiple of
 * trace_every (the reference's print rule, :682) and delivered to cb, in step
 * order, from the calling thread; device->host trace copies run on a side
 * stream while the next steps compute. */
int infoli_sim_run(infoli_sim* s, int n_steps, int trace_every, int trace_what, infoli_trace_cb cb,
                   void* user);

/* Same as infoli_sim_run, writing the trace rows into a caller buffer
 * out[rows][nq][n_cells] (nq = number of selected quantities); *rows_out
 * gets the row count.  out may be NULL when trace_every <= 0. */
int infoli_sim_run_into(infoli_sim* s, int n_steps, int trace_every, int trace_what, float* out,
                        int64_t out_capacity_floats, int* rows_out);

/* Copies the current state out / in ([INFOLI_NSTATE * n_cells] SoA). */
int infoli_sim_get_state(infoli_sim* s, float* state_out);
int infoli_sim_set_state(infoli_sim* s, const float* state_in);

/* Next step index (the reference's simStep). */
int infoli_sim_step(infoli_sim* s, int* step_out);

/* Kernel timing of the last infoli_sim_run (CUDA events on the launch
 * stream): total device milliseconds and number of kernel launches. */
int infoli_sim_last_run_stats(infoli_sim* s, float* device_ms, int* launches);

/* Plan summary: grid (CTAs), threads per CTA, total tiles, total chunks,
 * dynamic shared memory bytes. */
int infoli_sim_plan_info(infoli_sim* s, int* grid, int* threads, int* tiles, int* chunks,
                         int64_t* smem_bytes);

/* Device-side phase timers, the counterpart of the reference's -DPROFILING
 * build (src/hybrid/infoli.h:35-36, src/hybrid/infoli.c:637-643,974-1000),
 * which accumulates per-phase wall times.  When enabled, thread 0 of every
 * CTA accumulates global-timer intervals per step: [0] wait for the
 * neighbours' V_dend (tile staging / stamped words), [1] gap-junction
 * coupling, [2] voltage step (until the whole CTA is done), [3] grid barrier,
 * [4] gate units.  get_profile reports ns per step, averaged over CTAs
 * (mean_ns) and the slowest CTA (max_ns), since profiling was enabled. */
int infoli_sim_set_profiling(infoli_sim* s, int on);
int infoli_sim_get_profile(infoli_sim* s, double mean_ns[5], double max_ns[5]);

int infoli_sim_destroy(infoli_sim* s);

/* Asynchronous form of a run without trace (no counterpart in the
 * reference): enqueues n_steps steps on the simulation's own CUDA stream and
 * returns at once; the step counter advances immediately.  Simulations with
 * distinct handles run concurrently on the GPU when their grids fit side by
 * side.  infoli_sim_query returns 1 when all enqueued work has finished (0
 * while it runs, a negative status on a device error); infoli_sim_sync waits
 * for it.  get_state / set_state / run wait for enqueued work first. */
int infoli_sim_launch(infoli_sim* s, int n_steps);
/* Device memory the handle holds for its plan and state (bytes; trace
 * buffers and profiling timers excluded). */
int infoli_sim_memory(infoli_sim* s, int64_t* device_bytes);
int infoli_sim_query(infoli_sim* s);
int infoli_sim_sync(infoli_sim* s);

/* ------------------------------------------------------------------------ */
/* many independent networks in one launch                                   */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference, which simulates one network per process
 * (src/openmp/infoli.c:124-735); each network of a batch follows that
 * process's step (same parameters, same explicit-Euler update, the uniform
 * CONDUCTANCE of :320 as one conductance per network).  Networks are
 * independent: no coupling between them. */
typedef struct infoli_batch infoli_batch;

typedef struct {
  int n_nets;
  const int* n_cells;        /* [n_nets] cells per network, each <= 8192 */
  const float* params;       /* [INFOLI_NPARAM] shared by all networks */
  /* [INFOLI_NSTATE * total] SoA over the networks' cells laid end to end
   * (network 0's cells first), or NULL: broadcast init_values */
  const float* init_state;
  const float* init_values;  /* [INFOLI_NSTATE] */
  /* receiver bitmasks laid end to end: network i (n = n_cells[i], w =
   * ceil(n/32)) takes n * w words, row r = receiver r, bit s%32 of word s/32
   * = sender s (infoli_gen_bitmask's layout); self bits and bits >= n are
   * ignored */
  const uint32_t* bits;
  const float* g;            /* [n_nets] conductance of every edge of network i */
  int flags;                 /* INFOLI_F_KAHAN */
  int device;
  /* cells per CTA: 1024 (1,024-thread CTAs, clusters of up to 8) or 512
   * (512-thread CTAs, clusters of up to 16); 0 = the INFOLI_BATCH_SHAPE
   * environment variable (512), else 1024.  infoli_batch_autotune picks it
   * by measurement. */
  int block;
  /* which networks keep their bitmask rows in shared memory for the launch
   * (the rest stream them from L2/HBM every step):
   *   INFOLI_RES_FIT  every network whose rows fit in a CTA's shared memory
   *                   (the default);
   *   INFOLI_RES_OCC  only those whose rows fit while the CTAs per SM the
   *                   shape allows stay resident (two 512-thread CTAs per
   *                   SM; the same as INFOLI_RES_FIT for 1,024 threads);
   *   INFOLI_RES_NONE none.
   * infoli_batch_autotune picks it together with block. */
  int residency;
} infoli_batch_desc;

enum { INFOLI_RES_FIT = 0, INFOLI_RES_OCC = 1, INFOLI_RES_NONE = 2 };

/* Uploads the batch and packs it into thread-block clusters.  The stimulus
 * defaults to the reference's pulse (6 uA/cm2, steps 20000 to 20498) on every
 * cell of every network. */
int infoli_batch_create(const infoli_batch_desc* desc, infoli_batch** out);
int infoli_batch_set_stimulus_pulse(infoli_batch* b, int start_step, int end_step, float amp);
/* Advances every network by n_steps steps in one kernel launch (replayed
 * from a CUDA graph captured once per distinct n_steps); returns when done. */
int infoli_batch_run(infoli_batch* b, int n_steps);
/* out[INFOLI_NSTATE * total]: the state in init_state's layout. */
int infoli_batch_get_state(infoli_batch* b, float* out);
/* Replaces the state of every network (same layout); the step index and the
 * stimulus schedule are kept. */
int infoli_batch_set_state(infoli_batch* b, const float* in);
/* Launch shape and the device time of the last run (any pointer may be NULL). */
int infoli_batch_info(infoli_batch* b, int* ctas, int* cluster, int* block, int64_t* cells, float* last_ms);
/* Per CTA of the launch (arrays of `ctas` entries, any may be NULL): the
 * network it simulates (-1: idle slot of a cluster) and, for the last run,
 * its start and end times in ns from the earliest CTA start;
 * *max_active_clusters = clusters of this shape the device runs at once. */
int infoli_batch_cta_info(infoli_batch* b, int* max_active_clusters, int32_t* net, int64_t* start_ns,
                          int64_t* end_ns);
int infoli_batch_destroy(infoli_batch* b);

/* Autotuner of the batch's launch layout (no counterpart in the reference).
 * It times every candidate pair of cells per CTA and bitmask-row residency
 *   (1024, FIT), (1024, NONE), (512, FIT), (512, OCC), (512, NONE)
 * on a trial batch of a stratified sample of desc's networks (sorted by
 * size, evenly spaced, the fewest networks whose cells fill every SM twice
 * over at 1,024 cells per SM, at most max_sample when max_sample > 0, else at
 * most 4,096), with desc's flags, state and conductances: one run of
 * trial_steps steps to capture the graph, then the best of three timed runs.
 * It returns the pick in out->block and out->residency -- the first
 * candidate unless a later one is more than 2% faster than the pick so far
 * (trial noise is a few percent; the first candidate is the default layout)
 * -- and the device time per step of every candidate; pass both to
 * infoli_batch_create.  The trial steps start at step 0, so they see no
 * stimulus pulse.  desc itself is not modified. */
enum { INFOLI_TUNE_CANDIDATES = 5 };
typedef struct {
  int block;            /* the fastest candidate's cells per CTA: 1024 or 512 */
  int residency;        /* and its INFOLI_RES_* policy */
  int sample_nets;      /* networks in the trial batch */
  int64_t sample_cells; /* their cells */
  int cand_block[INFOLI_TUNE_CANDIDATES];
  int cand_residency[INFOLI_TUNE_CANDIDATES];
  float cand_ms_per_step[INFOLI_TUNE_CANDIDATES];  /* trial device time per step */
} infoli_batch_tune;
int infoli_batch_autotune(const infoli_batch_desc* desc, int max_sample, int trial_steps, infoli_batch_tune* out);
/* The autotuner's sample (host only, no GPU): writes the indices of the
 * sampled networks, in ascending order, to out_idx[n_nets] and returns their
 * count, or a negative status. */
int infoli_batch_tune_sample(int n_nets, const int* n_cells, int max_sample, int64_t target_cells, int* out_idx);

/* ------------------------------------------------------------------------ */
/* serving: a request loop over many simulations                             */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference (one network per process).  A server
 * admits simulation requests by device-memory budget, builds each one's plan
 * on a pool of host threads, runs admitted requests side by side on the GPU
 * and keeps their state on the device until they finish.  Requests that
 * arrive while others run start as soon as memory and SMs free up.
 *   - Small, light requests (at most 8,192 cells, one conductance, no
 *     repeated sender in a row, at most lane_edges_per_cta edges per CTA of
 *     their cluster) run in the lane: the batched cluster kernel over every
 *     such request on the device, relaunched every lane_chunk_steps steps; a
 *     request that arrives joins at the next launch and leaves when its
 *     steps are done.  A lane request runs on its own cluster of one CTA per
 *     1,024 cells, so only requests whose step that cluster keeps short take
 *     it.  The lane uses the SMs the other requests leave, and at least
 *     lane_sms of them.
 *   - Other requests each run their own persistent launch on their own
 *     stream, with a share of the SMs chosen from their size (at most all
 *     but lane_sms).
 * A request's result does not depend on the other requests: which path it
 * takes and its plan depend on the request alone. */
typedef struct infoli_server infoli_server;

typedef struct {
  const float* params;   /* [INFOLI_NPARAM] shared by all requests */
  int device;
  int64_t hbm_budget;    /* device bytes admitted requests may hold; 0 = 80% of free memory */
  int max_active;        /* requests admitted at once (preparing or running); 0 = 64 */
  int64_t work_per_cta;  /* edge evaluations per step per CTA when sizing a request's SM share; 0 = 32768 */
  int backfill_ms;       /* later requests may pass a head request that does not fit yet for this long; 0 = 1000 */
  int prep_threads;      /* host threads building plans; 0 = 4 */
  int flags;             /* INFOLI_F_KAHAN for every request */
  int age_ms;            /* prepared requests launch shortest estimated work (edges x steps) first;
                            one submitted this long ago goes ahead of them (oldest first); 0 = 10000,
                            < 0 = arrival order */
  int lane_sms;          /* SMs persistent requests leave to the lane; 0 = none kept back, < 0 = no lane */
  int lane_chunk_steps;  /* steps per lane launch (the join interval); 0 = 2000 */
  int lane_edges_per_cta;  /* lane eligibility: edges per CTA of the request's cluster at most this;
                              0 = 24576 (about 4 us of a lane step), < 0 = any */
} infoli_server_desc;

typedef struct {
  int n_cells;
  const int64_t* row_ptr;     /* CSR by receiver, as infoli_sim_desc */
  const int32_t* col;
  const float* g;             /* per-edge conductance or NULL */
  float g_uniform;
  const float* init_state;    /* [INFOLI_NSTATE * n_cells] or NULL */
  const float* init_values;   /* [INFOLI_NSTATE] when init_state is NULL */
  int n_steps;                /* simulated steps */
  int pulse_start, pulse_end; /* dendritic pulse of pulse_amp for pulse_start <= step < pulse_end */
  float pulse_amp;
} infoli_request_desc;

typedef struct {
  int64_t id;
  int n_cells, n_steps;
  int grid;                   /* CTAs (SMs) it ran on */
  int64_t device_bytes;       /* device memory it held */
  int64_t admitted_bytes;     /* budget reserved at admission (an estimate made before planning) */
  /* seconds since the server was created: submitted, admitted, plan and
   * upload done, launched, finished */
  double submit_s, admit_s, prepared_s, start_s, done_s;
  int status;                 /* INFOLI_OK or the request's error */
  double prep_start_s;        /* a preparation thread took it (admit_s .. prep_start_s: queued for one) */
  int lane;                   /* 1: ran in the lane (grid = its CTAs per lane launch) */
  int lane_launches;          /* lane launches it took part in */
} infoli_request_info;

int infoli_server_create(const infoli_server_desc* desc, infoli_server** out);
/* Copies the request's inputs and queues it; returns at once with its id.
 * INFOLI_ERR_CAPACITY when the request alone exceeds the budget. */
int infoli_server_submit(infoli_server* sv, const infoli_request_desc* req, int64_t* id);
/* 0 queued, 1 admitted or running, 2 finished. */
int infoli_server_poll(infoli_server* sv, int64_t id);
/* Waits for the request, copies its final state ([INFOLI_NSTATE * n_cells],
 * may be NULL) and timing, and forgets the id.  Returns the request's status. */
int infoli_server_wait(infoli_server* sv, int64_t id, float* out_state, infoli_request_info* info);
int infoli_server_status(infoli_server* sv, int* queued, int* active, int64_t* completed, int64_t* hbm_in_use);
/* Waits for running requests and drops queued ones. */
int infoli_server_destroy(infoli_server* sv);

/* ------------------------------------------------------------------------ */
/* allocation-free run                                                       */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference (its simulator allocates all of its own
 * memory).  For callers that must not allocate device memory: a host that
 * reserved a fixed device-memory arena at start-up and hands out only pieces
 * of it (an allocation outside the arena can fail or break its budget), a
 * language binding whose runtime's allocator owns every device buffer (memory
 * taken behind its back escapes its accounting), or a loop running beside
 * other GPU work, which cannot take the device-wide synchronisation that
 * cudaFree (and often cudaMalloc) implies.  This runs n_steps steps
 * without allocating anything: no cudaMalloc / cudaFree, no allocating
 * library call.  Everything is passed in device memory by the caller:
 *   d_row_ptr[n+1], d_col[E], d_g[E] or NULL (then g_uniform on every edge):
 *       CSR topology by receiver;
 *   d_state[INFOLI_NSTATE * n]: the 19 state arrays (SoA, bin/default.conf
 *       order), read at the start and overwritten with the state after the
 *       run;
 *   d_trace_axon[n_steps * n] or NULL: V_axon after every step.
 * The stimulus is one global pulse (pulse_amp for pulse_start <= step <
 * pulse_end; the reference's default is 20000, 20499, 6).  step0 is the index
 * of the first step; step0 + n_steps must not exceed INT_MAX.  `stream` is a
 * cudaStream_t (NULL: the default stream); the call returns after the run has
 * finished on it, having synchronised that stream only.
 * Topology contract: d_row_ptr[0..n] non-decreasing from d_row_ptr[0] >= 0,
 * and d_row_ptr[n] no larger than the length of d_col and d_g.  A decreasing
 * or negative row_ptr, a sender id outside [0, n) or a NULL d_col with edges
 * is detected on the device, skipped without reading outside the arrays, and
 * returned as INFOLI_ERR_ARG; d_row_ptr[n] beyond the caller's arrays cannot
 * be detected.
 * Precision between calls: Ca2Plus is carried in FP64 on the device during a
 * call but d_state holds FP32, so each call ends by rounding it to FP32.  Two
 * chained calls therefore differ from one call of the same total length in
 * the last bits of Ca2Plus (and what follows from them), unlike
 * infoli_sim_run, which keeps the FP64 value between runs.
 * Device waits (the grid barrier) give up after INFOLI_WAIT_TIMEOUT_MS
 * (default 4000 ms) and return INFOLI_ERR_TIMEOUT.
 * The only scratch (V_dend double buffer, barrier counter, error word) is a
 * static device array of fixed size in the library, so networks are limited
 * to 65536 cells (INFOLI_ERR_CAPACITY beyond).  Every GPU that loads the
 * library holds that array (about 0.5 MiB) until the process exits.  The
 * first call on a device looks up the array's device address (with that
 * device current): make that first call before any stream capture.  All
 * calls share the array, so calls that overlap on the GPU (different
 * streams, threads or processes sharing a context) race and must be
 * serialised by the caller. */
int infoli_run_noalloc(const float* params, int n_cells, const int64_t* d_row_ptr, const int32_t* d_col,
                       const float* d_g, float g_uniform, int pulse_start, int pulse_end, float pulse_amp,
                       float* d_state, int step0, int n_steps, float* d_trace_axon, void* stream);

/* Host-side check of the work planner (no GPU needed; no counterpart in the
 * reference): plans an n-cell network for a device with grid_max co-resident
 * CTAs of `threads` threads and smem_budget bytes of shared memory per CTA
 * (sync_mode 0 auto, 1 grid barrier, 2 stamped words; grid 0 = automatic),
 * then computes the gap-junction currents of the voltages vdend[n] by walking
 * the plan's tables with the step kernel's addressing, every shared-memory
 * offset bounds-checked.  info[10] = {CTAs, stamped, tiles (stamped plans: 1
 * when the planner relabelled the cells), chunks or groups, partial slots,
 * shared bytes, progress probes, resident, shared-memory wavefronts of the
 * stamped V_dend gathers, gather instructions}.  vdend and ic_out are in the
 * caller's cell order either way.  Returns 0 or a negative code naming the
 * violated invariant. */
int infoli_plan_emulate(int n, const int64_t* row_ptr, const int32_t* col, const float* g, float g_uniform,
                        int grid, int grid_max, int threads, int64_t smem_budget, int sync_mode,
                        const float* vdend, float* ic_out, int64_t info[10]);

/* The planner's locality-preserving cell order (no counterpart in the
 * reference).  Stamped plans whose windows are wide are re-planned in this
 * order: spectral coordinates of the cells (the two lowest non-trivial
 * eigenvectors of the in-edge graph Laplacian) cut into `parts` compact
 * blocks of at most `threads` cells by recursive coordinate bisection.
 * order[new] = old cell id, starts[parts + 1] = the blocks in the new order.
 * The caller's cell order stays the order of every array at this interface.
 * Returns 0, or -1 when no such order exists (e.g. too few cells). */
int infoli_plan_locality_order(int n, const int64_t* row_ptr, const int32_t* col, int parts, int threads,
                               int32_t* order, int32_t* starts);

/* ------------------------------------------------------------------------ */
/* trace text (host side)                                                    */
/* ------------------------------------------------------------------------ */

/* "%.8f" of one float (promoted to double), byte-identical to the C
 * library's printf; out needs 64 bytes.  Returns the length. */
int infoli_format_f8(char* out, float v);

/* One row of the reference's trace file (src/openmp/infoli.c:684-695):
 * tagged != 0 gives "%d : %.8f " per cell with 1-based ids (normal build),
 * tagged == 0 gives "%.8f " per cell (regression build); then "\n".
 * Formats with up to nthreads threads (<= 0: all).  Returns bytes written or
 * -1 when cap is too small (40 * n + 2 bytes always suffice). */
int64_t infoli_format_row(char* buf, int64_t cap, const float* values, int n, int tagged, int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* INFOLI_GPU_H */
