// C ABI of libinfoli_gpu.so: simulation handles, device memory, the chunked
// launch loop and trace streaming (pinned host slots filled by
// cudaMemcpyAsync on a side stream while the next chunk of steps computes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/infoli_gpu.h"
#include "infoli_internal.h"
#include "infoli_kernels.cuh"
#include "infoli_planner.h"

using namespace infoli;

extern "C" unsigned long long infoli__wait_timeout_ns(void) {
  const char* s = getenv("INFOLI_WAIT_TIMEOUT_MS");
  long ms = s ? atol(s) : 4000;
  if (ms <= 0) ms = 4000;
  return (unsigned long long)ms * 1000000ull;
}

#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return infoli__fail(INFOLI_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                          __FILE__, __LINE__);                                                      \
  } while (0)

namespace {

constexpr int kThreads = 1024;
constexpr int kMaxStepsPerLaunch = 8192;
constexpr size_t kTraceSlotBytes = 64u << 20;

// Device memory of simulation handles comes from one stream-ordered pool per
// device (cudaMallocFromPoolAsync / cudaFreeAsync on the handle's stream).
// Plain cudaMalloc / cudaFree synchronise with work already running on the
// device, so creating or destroying one handle would stall the kernels of
// every other handle; stream-ordered allocation does not.  Freed memory stays
// in the pool for the next handle (release threshold: unlimited).
cudaMemPool_t sim_pool(int device);

}  // namespace

extern "C" cudaMemPool_t infoli__device_pool(int device) { return sim_pool(device); }

namespace {

cudaMemPool_t sim_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (device < 0 || device >= 64) return nullptr;
  if (!pools[device]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&pools[device], &props) != cudaSuccess) {
      pools[device] = nullptr;
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pools[device], cudaMemPoolAttrReleaseThreshold, &keep);
  }
  return pools[device];
}

template <class T>
cudaError_t pool_alloc(T** dst, size_t bytes, int device, cudaStream_t st) {
  cudaMemPool_t pool = sim_pool(device);
  if (!pool) return cudaErrorMemoryAllocation;
  return cudaMallocFromPoolAsync((void**)dst, bytes, pool, st);
}

template <class T>
int dev_upload(T** dst, const T* src, size_t count, int device, cudaStream_t st) {
  *dst = nullptr;
  if (count == 0) return INFOLI_OK;
  CK(pool_alloc(dst, count * sizeof(T), device, st));
  CK(cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, st));
  return INFOLI_OK;
}

}  // namespace

struct infoli_sim {
  int device = 0;
  int n = 0;
  int n_pad = 0;
  ModelParams P{};
  float g_uniform = 0.04f;
  int kahan = 0;
  int step = 0;
  // plan
  Plan plan;
  CtaWork* d_cta = nullptr;
  TileDesc* d_tiles = nullptr;
  ChunkDesc* d_chunks = nullptr;
  CellSlots* d_cell_slots = nullptr;
  uint16_t* d_edges = nullptr;
  float* d_edge_g = nullptr;
  int* d_probes = nullptr;
  int2_t* d_gdesc = nullptr;
  int32_t* d_gcol = nullptr;  // gather plans; stamped plans: window sender ids
  int32_t* d_perm = nullptr;  // relabelled plans: caller's cell id of each plan cell
  unsigned long long* d_vll[2] = {nullptr, nullptr};  // stamped exchange words
  float* d_vds[2] = {nullptr, nullptr};               // bitmask plans: scaled V_dend
  // state
  float* d_vd[2] = {nullptr, nullptr};
  float* d_st = nullptr;
  double* d_ca = nullptr;
  float* d_io = nullptr;  // the C ABI's 19 x n state layout, staged on the device
  // stimulus
  int stim_kind = STIM_PULSE;
  int stim_start = 20000, stim_end = 20499;
  float stim_amp = 6.0f;
  float* d_cell_amp = nullptr;
  int* d_cell_onset = nullptr;
  int stim_dur = 0;
  float* d_stim_table = nullptr;  // STIM_TABLE: [stim_rows][n_pad]
  int stim_rows = 0, stim_first = 0;
  // sync
  unsigned* d_bar = nullptr;
  int* d_err = nullptr;
  unsigned long long* d_prof = nullptr;  // per-CTA phase timers when profiling is on
  // trace ring
  float* d_trace[2] = {nullptr, nullptr};
  float* h_trace[2] = {nullptr, nullptr};
  size_t trace_slot_floats = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t ev_kernel[2] = {nullptr, nullptr}, ev_copy[2] = {nullptr, nullptr};
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
  float last_ms = 0.0f;
  int last_launches = 0;
  int async_pending = 0;  // infoli_sim_launch work not yet checked for device errors
  int64_t dev_bytes = 0;  // device memory held for the plan and the state
};

namespace {

void release(infoli_sim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->side) cudaStreamSynchronize(s->side);
  void* dptrs[] = {s->d_cta,   s->d_tiles,  s->d_chunks, s->d_cell_slots, s->d_edges,
                   s->d_edge_g, s->d_vd[0], s->d_vd[1],  s->d_st,         s->d_ca,
                   s->d_cell_amp, s->d_cell_onset, s->d_bar, s->d_err, s->d_trace[0], s->d_trace[1],
                   s->d_prof, s->d_probes, s->d_vll[0], s->d_vll[1], s->d_gdesc, s->d_stim_table,
                   s->d_gcol, s->d_perm, s->d_io, s->d_vds[0], s->d_vds[1]};
  if (s->stream) {
    for (void* p : dptrs)
      if (p) cudaFreeAsync(p, s->stream);
    cudaStreamSynchronize(s->stream);
  }
  for (float* h : s->h_trace)
    if (h) cudaFreeHost(h);
  for (cudaEvent_t e : {s->ev_kernel[0], s->ev_kernel[1], s->ev_copy[0], s->ev_copy[1], s->ev_t0, s->ev_t1})
    if (e) cudaEventDestroy(e);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->side) cudaStreamDestroy(s->side);
  delete s;
}

// Map the 19 reference state arrays to device fields.
const int kFieldOfState[INFOLI_NSTATE] = {
    -1 /*V_dend -> vd*/, F_R, F_S, F_Q, -2 /*Ca2Plus -> ca*/, F_ICAH, F_GCAL, F_VS, F_M, F_H, F_N, F_P,
    F_XS, F_K, F_L, F_VA, F_MA, F_HA, F_XA};

struct StateMap {
  int field[INFOLI_NSTATE];
};

// ABI layout (19 x n floats, reference order) <-> device layout (F_COUNT x
// n_pad floats, FP64 Ca2+, V_dend in both halves of its double buffer).
// One thread per (array, cell); padding cells stay as they are.
__global__ void state_scatter_kernel(const float* __restrict__ in, int n, long long np, StateMap m, float* st,
                                     double* ca, float* vd0, float* vd1) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)INFOLI_NSTATE * n) return;
  const int k = (int)(i / n), c = (int)(i - (long long)k * n);
  const float v = in[i];
  const int f = m.field[k];
  if (f == -1) {
    vd0[c] = v;
    vd1[c] = v;
  } else if (f == -2) {
    ca[c] = (double)v;
  } else {
    st[(long long)f * np + c] = v;
  }
}

__global__ void state_gather_kernel(float* __restrict__ out, int n, long long np, StateMap m, const float* st,
                                    const double* ca, const float* vd) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)INFOLI_NSTATE * n) return;
  const int k = (int)(i / n), c = (int)(i - (long long)k * n);
  const int f = m.field[k];
  out[i] = f == -1 ? vd[c] : f == -2 ? (float)ca[c] : st[(long long)f * np + c];
}

StateMap state_map() {
  StateMap m;
  for (int k = 0; k < INFOLI_NSTATE; ++k) m.field[k] = kFieldOfState[k];
  return m;
}

int state_io_buffer(infoli_sim* s) {
  if (s->d_io) return INFOLI_OK;
  return pool_alloc(&s->d_io, (size_t)INFOLI_NSTATE * s->n * sizeof(float), s->device, s->stream) == cudaSuccess
             ? INFOLI_OK
             : infoli__fail(INFOLI_ERR_NOMEM, "state staging buffer: device allocation failed");
}

// One host->device copy of the caller's 19 x n array (a direct DMA when the
// caller's buffer is pinned), then the scatter on the device.  Returns after
// the copy has completed, so the caller may reuse its buffer.
int upload_state(infoli_sim* s, const float* state /*19 x n*/) {
  const int n = s->n;
  const long long total = (long long)INFOLI_NSTATE * n;
  if (int rc = state_io_buffer(s)) return rc;
  CK(cudaMemcpyAsync(s->d_io, state, (size_t)total * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  state_scatter_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s->stream>>>(
      s->d_io, n, (long long)s->n_pad, state_map(), s->d_st, s->d_ca, s->d_vd[s->step & 1],
      s->d_vd[(s->step + 1) & 1]);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s->stream));
  return INFOLI_OK;
}

// The same at creation, by copies only: the state is repacked on the host
// (19 x n floats -> the device's field rows, FP64 Ca2+, V_dend in both halves
// of its double buffer) and moved with one copy per array on the copy
// engines.  A kernel here would wait for free SMs while other simulations'
// persistent grids hold them all, which made a serving request's preparation
// wait for the running requests.  Padding cells stay as they are, as with
// the scatter.
int upload_state_copies(infoli_sim* s, const float* state /*19 x n*/) {
  const int n = s->n;
  const size_t np = (size_t)s->n_pad;
  std::vector<double> ca((size_t)n);
  for (int k = 0; k < INFOLI_NSTATE; ++k) {
    const float* src = state + (size_t)k * n;
    const int f = kFieldOfState[k];
    if (f == -1) {
      CK(cudaMemcpyAsync(s->d_vd[s->step & 1], src, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
      CK(cudaMemcpyAsync(s->d_vd[(s->step + 1) & 1], src, (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                         s->stream));
    } else if (f == -2) {
      for (int c = 0; c < n; ++c) ca[(size_t)c] = (double)src[c];
      CK(cudaMemcpyAsync(s->d_ca, ca.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    } else {
      CK(cudaMemcpyAsync(s->d_st + (size_t)f * np, src, (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                         s->stream));
    }
  }
  CK(cudaStreamSynchronize(s->stream));
  return INFOLI_OK;
}

int fill_args(infoli_sim* s, StepArgs* a) {
  std::memset(a, 0, sizeof *a);
  a->P = s->P;
  a->cta = s->d_cta;
  a->tiles = s->d_tiles;
  a->chunks = s->d_chunks;
  a->cell_slots = reinterpret_cast<const int2*>(s->d_cell_slots);
  a->edges = s->d_edges;
  a->edge_g = s->d_edge_g;
  a->cell_g = nullptr;
  a->g_uniform = s->g_uniform;
  a->vd[0] = s->d_vd[0];
  a->vd[1] = s->d_vd[1];
  a->st = s->d_st;
  a->ca = s->d_ca;
  a->n_pad = s->n_pad;
  a->stim_kind = s->stim_kind;
  a->stim_start = s->stim_start;
  a->stim_end = s->stim_end;
  a->stim_amp = s->stim_amp;
  a->cell_amp = s->d_cell_amp;
  a->cell_onset = s->d_cell_onset;
  a->stim_dur = s->stim_dur;
  a->bar = s->d_bar;
  a->err = s->d_err;
  a->timeout_ns = infoli__wait_timeout_ns();
  // failure-detection test hook (see StepArgs::stall_cta); unset in normal use
  const char* stall = getenv("INFOLI_STALL_CTA");
  a->stall_cta = stall ? atoi(stall) : -1;
  a->shape = s->plan.shape;
  a->prof = s->d_prof;
  a->vll[0] = s->d_vll[0];
  a->vll[1] = s->d_vll[1];
  a->vds[0] = s->d_vds[0];
  a->vds[1] = s->d_vds[1];
  a->probes = s->d_probes;
  a->gdesc = reinterpret_cast<const int2*>(s->d_gdesc);
  a->gcol = s->d_gcol;
  a->perm = s->d_perm;
  a->n_cells = s->n;
  return INFOLI_OK;
}

int count_rows(int step0, int n_steps, int every) {
  if (every <= 0 || n_steps <= 0) return 0;
  // multiples of `every` in [step0, step0 + n_steps)
  const long long hi = (long long)step0 + n_steps - 1;
  const long long first = ((long long)step0 + every - 1) / every;
  const long long last = hi / every;
  return last >= first ? (int)(last - first + 1) : 0;
}

int nq_of(int what) { return !!(what & INFOLI_TRACE_AXON) + !!(what & INFOLI_TRACE_SOMA) + !!(what & INFOLI_TRACE_DEND); }

int check_device_error(infoli_sim* s) {
  int err = 0;
  CK(cudaMemcpyAsync(&err, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (err != DEV_OK) {
    cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream);
    return infoli__fail(INFOLI_ERR_TIMEOUT, "device wait gave up (code %d): %s", err,
                        err == DEV_ERR_BARRIER_TIMEOUT ? "grid barrier timeout"
                        : err == DEV_ERR_STAMP_TIMEOUT ? "stamped V_dend exchange timeout"
                                                       : "tile copy timeout");
  }
  return INFOLI_OK;
}

}  // namespace

extern "C" {

const char* infoli_build_info(void) {
  return "libinfoli_gpu: sm_103a persistent cooperative step kernel, bulk-async (TMA) V_dend tiles, "
         "FP32 coupling with SFU exp2, FP64 Ca2+";
}

int infoli_device_count(void) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  return n;
}

int infoli_sim_create(const infoli_sim_desc* d, infoli_sim** out) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_sim_create");
  if (!d || !out) return infoli__fail(INFOLI_ERR_ARG, "sim_create: null argument");
  *out = nullptr;
  if (d->n_cells <= 0) return infoli__fail(INFOLI_ERR_ARG, "sim_create: n_cells must be positive");
  if (!d->params) return infoli__fail(INFOLI_ERR_ARG, "sim_create: params is NULL");
  if (!d->init_state && !d->init_values)
    return infoli__fail(INFOLI_ERR_ARG, "sim_create: need init_state or init_values");
  if (!d->row_ptr) return infoli__fail(INFOLI_ERR_ARG, "sim_create: row_ptr is NULL");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return infoli__fail(INFOLI_ERR_CUDA, "sim_create: no CUDA device available");
  if (d->device < 0 || d->device >= ndev) return infoli__fail(INFOLI_ERR_ARG, "sim_create: bad device %d", d->device);

  infoli_sim* s = new infoli_sim();
  s->device = d->device;
  s->n = d->n_cells;
  s->n_pad = pad_cells(d->n_cells);
  s->g_uniform = d->g_uniform;
  s->kahan = (d->flags & INFOLI_F_KAHAN) ? 1 : 0;
  static_assert(sizeof(ModelParams) == INFOLI_NPARAM * sizeof(float), "param layout");
  std::memcpy(&s->P, d->params, sizeof(ModelParams));

  auto fail = [&](int rc) {
    release(s);
    return rc;
  };
  if (cudaSetDevice(s->device) != cudaSuccess) return fail(infoli__fail(INFOLI_ERR_CUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_CUDA, "stream creation failed"));

  // ---- plan
  int nsm = 0, smem_optin = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, s->device);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device);
  PlanInput pin;
  pin.n = s->n;
  pin.row_ptr = d->row_ptr;
  pin.col = d->col;
  pin.g = d->g;
  pin.grid = 0;
  const char* gs = getenv("INFOLI_GRID");
  if (gs) pin.grid = atoi(gs);
  pin.grid_max = nsm;  // one CTA per SM
  if (d->grid > 0) pin.grid_max = std::min(nsm, d->grid);  // a share of the SMs
  pin.smem_budget = (size_t)smem_optin - 1024;  // static shared (abort flag) headroom
  pin.kahan = s->kahan;
  pin.no_resident = getenv("INFOLI_NO_RESIDENT") ? 1 : 0;
  pin.reorder = getenv("INFOLI_NO_REORDER") ? 0 : 1;
  if (const char* sm = getenv("INFOLI_SYNC"))
    pin.sync_mode = !strcmp(sm, "barrier")   ? kSyncBarrier
                    : !strcmp(sm, "stamped") ? kSyncStamped
                    : !strcmp(sm, "gather")  ? kSyncGather
                    : !strcmp(sm, "tgather") ? kSyncTiledGather
                    : !strcmp(sm, "bits")    ? kSyncBits
                                             : kSyncAuto;
  // 512-thread CTAs (128 registers per thread) whenever the network fits in
  // one cell per thread at that size; 1024 threads for larger networks.
  // INFOLI_THREADS=512|1024 overrides.
  int want_threads = 0;
  if (const char* ts = getenv("INFOLI_THREADS")) want_threads = atoi(ts) == 512 ? 512 : 1024;
  std::string perr;
  bool planned = false;
  for (int threads : {512, kThreads}) {
    if (want_threads && threads != want_threads) continue;
    if (!want_threads && threads == 512 && (int64_t)nsm * 512 < s->n) continue;
    pin.threads = threads;
    if (make_plan(pin, &s->plan, &perr)) {
      planned = true;
      break;
    }
  }
  // plans with one thread per receiver (gather, tiled gather, bitmask) hide
  // their load latency with more warps: 1024-thread CTAs when the choice is free
  if (planned && !want_threads && s->plan.shape.gather && s->plan.threads == 512) {
    Plan wide;
    pin.threads = kThreads;
    if (make_plan(pin, &wide, &perr) && wide.shape.gather == s->plan.shape.gather) s->plan = std::move(wide);
  }
  if (!planned) return fail(infoli__fail(INFOLI_ERR_ARG, "%s", perr.c_str()));
  cudaError_t occ_err = cudaSuccess;
  const int cores = max_coresident_ctas(s->plan.threads, s->plan.smem_bytes, &occ_err);
  if (cores < s->plan.grid)
    return fail(infoli__fail(INFOLI_ERR_CUDA, "plan needs %d co-resident CTAs of %d threads and %lld bytes of shared "
                             "memory, device allows %d (%s)", s->plan.grid, s->plan.threads,
                             (long long)s->plan.smem_bytes, cores, cudaGetErrorString(occ_err)));

  int rc;
  const int dv = s->device;
  cudaStream_t st0 = s->stream;
  if ((rc = dev_upload(&s->d_cta, s->plan.cta.data(), s->plan.cta.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_tiles, s->plan.tiles.data(), s->plan.tiles.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_chunks, s->plan.chunks.data(), s->plan.chunks.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_cell_slots, s->plan.cell_slots.data(), s->plan.cell_slots.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_edges, s->plan.edges.data(), s->plan.edges.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_edge_g, s->plan.edge_g.data(), s->plan.edge_g.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_probes, s->plan.probes.data(), s->plan.probes.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_gdesc, s->plan.gdesc.data(), s->plan.gdesc.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_gcol, s->plan.gcol.data(), s->plan.gcol.size(), dv, st0)) ||
      (rc = dev_upload(&s->d_perm, s->plan.perm.data(), s->plan.perm.size(), dv, st0)))
    return fail(rc);
  // the kernel needs valid pointers even for empty tables
  if ((!s->d_chunks && pool_alloc(&s->d_chunks, sizeof(ChunkDesc), dv, st0) != cudaSuccess) ||
      (!s->d_tiles && pool_alloc(&s->d_tiles, sizeof(TileDesc), dv, st0) != cudaSuccess) ||
      (!s->d_edges && pool_alloc(&s->d_edges, 16, dv, st0) != cudaSuccess))
    return fail(infoli__fail(INFOLI_ERR_NOMEM, "sim_create: device allocation failed"));

  const size_t np = (size_t)s->n_pad;
  if (pool_alloc(&s->d_vd[0], np * sizeof(float), dv, st0) != cudaSuccess ||
      pool_alloc(&s->d_vd[1], np * sizeof(float), dv, st0) != cudaSuccess ||
      pool_alloc(&s->d_st, (size_t)F_COUNT * np * sizeof(float), dv, st0) != cudaSuccess ||
      pool_alloc(&s->d_ca, np * sizeof(double), dv, st0) != cudaSuccess ||
      pool_alloc(&s->d_bar, 128, dv, st0) != cudaSuccess || pool_alloc(&s->d_err, 128, dv, st0) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_NOMEM, "sim_create: device allocation failed"));
  cudaMemsetAsync(s->d_vd[0], 0, np * sizeof(float), st0);
  cudaMemsetAsync(s->d_vd[1], 0, np * sizeof(float), st0);
  cudaMemsetAsync(s->d_err, 0, 128, st0);
  cudaMemsetAsync(s->d_bar, 0, 128, st0);
  if (s->plan.shape.stamped) {
    if (pool_alloc(&s->d_vll[0], np * sizeof(unsigned long long), dv, st0) != cudaSuccess ||
        pool_alloc(&s->d_vll[1], np * sizeof(unsigned long long), dv, st0) != cudaSuccess)
      return fail(infoli__fail(INFOLI_ERR_NOMEM, "sim_create: device allocation failed"));
  }
  if (s->plan.shape.gather == 3) {
    if (pool_alloc(&s->d_vds[0], np * sizeof(float), dv, st0) != cudaSuccess ||
        pool_alloc(&s->d_vds[1], np * sizeof(float), dv, st0) != cudaSuccess)
      return fail(infoli__fail(INFOLI_ERR_NOMEM, "sim_create: device allocation failed"));
    cudaMemsetAsync(s->d_vds[0], 0, np * sizeof(float), st0);
    cudaMemsetAsync(s->d_vds[1], 0, np * sizeof(float), st0);
  }

  std::vector<float> init;
  const float* st = d->init_state;
  if (!st) {
    init.resize((size_t)INFOLI_NSTATE * s->n);
    for (int k = 0; k < INFOLI_NSTATE; ++k)
      std::fill(init.begin() + (size_t)k * s->n, init.begin() + (size_t)(k + 1) * s->n, d->init_values[k]);
    st = init.data();
  }
  if ((rc = upload_state_copies(s, st))) return fail(rc);
  for (int i = 0; i < 2; ++i)
    if (cudaEventCreateWithFlags(&s->ev_kernel[i], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_copy[i], cudaEventDisableTiming) != cudaSuccess)
      return fail(infoli__fail(INFOLI_ERR_CUDA, "event creation failed"));
  if (cudaEventCreate(&s->ev_t0) != cudaSuccess || cudaEventCreate(&s->ev_t1) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_CUDA, "event creation failed"));
  const Plan& pl = s->plan;
  s->dev_bytes = (int64_t)(pl.cta.size() * sizeof(CtaWork) + pl.tiles.size() * sizeof(TileDesc) +
                           pl.chunks.size() * sizeof(ChunkDesc) + pl.cell_slots.size() * sizeof(CellSlots) +
                           pl.edges.size() * sizeof(uint16_t) + pl.edge_g.size() * sizeof(float) +
                           pl.probes.size() * sizeof(int) + pl.gdesc.size() * sizeof(int2_t) +
                           pl.gcol.size() * sizeof(int32_t)) +
                 (int64_t)np * (2 * sizeof(float) + F_COUNT * sizeof(float) + sizeof(double)) + 256 +
                 (pl.shape.stamped ? (int64_t)np * 2 * sizeof(unsigned long long) : 0);
  *out = s;
  return INFOLI_OK;
}

int infoli_sim_memory(infoli_sim* s, int64_t* device_bytes) {
  infoli__clear_error();
  if (!s || !device_bytes) return infoli__fail(INFOLI_ERR_ARG, "sim_memory: bad argument");
  *device_bytes = s->dev_bytes;
  return INFOLI_OK;
}

int infoli_sim_destroy(infoli_sim* s) {
  infoli__clear_error();
  release(s);
  return INFOLI_OK;
}

int infoli_sim_set_stimulus_pulse(infoli_sim* s, int start_step, int end_step, float amp) {
  infoli__clear_error();
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  s->stim_kind = STIM_PULSE;
  s->stim_start = start_step;
  s->stim_end = end_step;
  s->stim_amp = amp;
  return INFOLI_OK;
}

int infoli_sim_set_stimulus_cells(infoli_sim* s, const float* amp, const int* onset, int duration) {
  infoli__clear_error();
  if (!s || !amp || !onset || duration < 0) return infoli__fail(INFOLI_ERR_ARG, "set_stimulus_cells: bad argument");
  CK(cudaSetDevice(s->device));
  if (!s->d_cell_amp) {
    CK(pool_alloc(&s->d_cell_amp, (size_t)s->n_pad * sizeof(float), s->device, s->stream));
    CK(pool_alloc(&s->d_cell_onset, (size_t)s->n_pad * sizeof(int), s->device, s->stream));
    CK(cudaMemsetAsync(s->d_cell_amp, 0, (size_t)s->n_pad * sizeof(float), s->stream));
    CK(cudaMemsetAsync(s->d_cell_onset, 0, (size_t)s->n_pad * sizeof(int), s->stream));
  }
  CK(cudaMemcpyAsync(s->d_cell_amp, amp, (size_t)s->n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(s->d_cell_onset, onset, (size_t)s->n * sizeof(int), cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->stim_kind = STIM_CELL;
  s->stim_dur = duration;
  return INFOLI_OK;
}

int infoli_sim_set_stimulus_table(infoli_sim* s, const float* table, int rows, int first_step) {
  infoli__clear_error();
  if (!s || !table || rows <= 0) return infoli__fail(INFOLI_ERR_ARG, "set_stimulus_table: bad argument");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  if (s->d_stim_table) cudaFreeAsync(s->d_stim_table, s->stream);
  s->d_stim_table = nullptr;
  const size_t np = (size_t)s->n_pad;
  CK(pool_alloc(&s->d_stim_table, (size_t)rows * np * sizeof(float), s->device, s->stream));
  CK(cudaMemsetAsync(s->d_stim_table, 0, (size_t)rows * np * sizeof(float), s->stream));
  CK(cudaMemcpy2DAsync(s->d_stim_table, np * sizeof(float), table, (size_t)s->n * sizeof(float),
                       (size_t)s->n * sizeof(float), (size_t)rows, cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->stim_kind = STIM_TABLE;
  s->stim_rows = rows;
  s->stim_first = first_step;
  return INFOLI_OK;
}

namespace {
// A table stimulus covers [stim_first, stim_first + stim_rows); runs stay inside.
int check_table_range(const infoli_sim* s, int n_steps) {
  if (s->stim_kind != STIM_TABLE) return INFOLI_OK;
  if (s->step < s->stim_first || (long long)s->step + n_steps > (long long)s->stim_first + s->stim_rows)
    return infoli__fail(INFOLI_ERR_ARG, "run of steps %d..%lld leaves the stimulus table (steps %d..%lld)", s->step,
                        (long long)s->step + n_steps - 1, s->stim_first, (long long)s->stim_first + s->stim_rows - 1);
  return INFOLI_OK;
}
const float* table_at(const infoli_sim* s, int step0) {
  return s->stim_kind == STIM_TABLE ? s->d_stim_table + (size_t)(step0 - s->stim_first) * s->n_pad : nullptr;
}
}  // namespace

int infoli_sim_run(infoli_sim* s, int n_steps, int trace_every, int trace_what, infoli_trace_cb cb, void* user) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_sim_run");
  if (!s || n_steps < 0) return infoli__fail(INFOLI_ERR_ARG, "sim_run: bad argument");
  if (trace_every > 0 && (!cb || nq_of(trace_what) == 0))
    return infoli__fail(INFOLI_ERR_ARG, "sim_run: tracing needs a callback and at least one quantity");
  CK(cudaSetDevice(s->device));
  if (int rc0 = check_table_range(s, n_steps)) return rc0;
  const int nq = trace_every > 0 ? nq_of(trace_what) : 0;
  const size_t row_floats = (size_t)nq * s->n_pad;

  // launch length: bounded by kMaxStepsPerLaunch and by the trace slot size
  int launch_steps = std::min(std::max(n_steps, 1), kMaxStepsPerLaunch);
  if (nq > 0) {
    const int rows_cap = (int)std::max<size_t>(1, kTraceSlotBytes / (row_floats * sizeof(float)));
    launch_steps = std::min<long long>(launch_steps, (long long)rows_cap * trace_every);
    const size_t need = (size_t)rows_cap * row_floats;
    const int rows_needed = count_rows(0, launch_steps + trace_every, trace_every) + 1;
    const size_t want = std::min(need, (size_t)rows_needed * row_floats);
    if (s->trace_slot_floats < want) {
      CK(cudaStreamSynchronize(s->stream));
      for (int i = 0; i < 2; ++i) {
        if (s->d_trace[i]) cudaFreeAsync(s->d_trace[i], s->stream);
        if (s->h_trace[i]) cudaFreeHost(s->h_trace[i]);
        s->d_trace[i] = nullptr;
        s->h_trace[i] = nullptr;
      }
      for (int i = 0; i < 2; ++i) {
        CK(pool_alloc(&s->d_trace[i], want * sizeof(float), s->device, s->stream));
        CK(cudaMallocHost((void**)&s->h_trace[i], want * sizeof(float)));
      }
      s->trace_slot_floats = want;
    }
  }

  StepArgs a;
  fill_args(s, &a);
  a.trace_every = trace_every > 0 ? trace_every : 0;
  a.trace_mask = trace_what;
  a.trace_nq = nq;

  struct Pending {
    int slot, step0, rows;
  };
  std::vector<Pending> pend;
  int launches = 0;
  CK(cudaEventRecord(s->ev_t0, s->stream));
  int done = 0, li = 0;
  auto drain = [&](const Pending& p) -> int {
    CK(cudaEventSynchronize(s->ev_copy[p.slot]));
    // rows are the multiples of trace_every in the launch's step range
    int st = ((p.step0 + trace_every - 1) / trace_every) * trace_every;
    for (int row = 0; row < p.rows; ++row, st += trace_every) {
      const float* base = s->h_trace[p.slot] + (size_t)row * row_floats;
      int qi = 0;
      for (int bit : {INFOLI_TRACE_AXON, INFOLI_TRACE_SOMA, INFOLI_TRACE_DEND})
        if (trace_what & bit) cb(user, st, bit, base + (size_t)(qi++) * s->n_pad, s->n);
    }
    return INFOLI_OK;
  };
  while (done < n_steps) {
    const int len = std::min(launch_steps, n_steps - done);
    const int slot = li & 1;
    a.step0 = s->step + done;
    a.n_steps = len;
    a.stim_table = table_at(s, a.step0);
    a.trace = nq ? s->d_trace[slot] : nullptr;
    const int rows = count_rows(a.step0, len, trace_every);
    // the slot's previous contents must have been copied and consumed
    if (pend.size() >= 2) {
      int rc = drain(pend.front());
      if (rc) return rc;
      pend.erase(pend.begin());
    }
    CK(cudaMemsetAsync(s->d_bar, 0, sizeof(unsigned), s->stream));
    if (s->plan.shape.stamped) {  // no stale stamp may match a step of this launch
      CK(cudaMemsetAsync(s->d_vll[0], 0xff, (size_t)s->n_pad * sizeof(unsigned long long), s->stream));
      CK(cudaMemsetAsync(s->d_vll[1], 0xff, (size_t)s->n_pad * sizeof(unsigned long long), s->stream));
    }
    CK(launch_step_kernel(a, s->plan.grid, s->plan.threads, s->stream));
    ++launches;
    if (rows > 0) {
      CK(cudaEventRecord(s->ev_kernel[slot], s->stream));
      CK(cudaStreamWaitEvent(s->side, s->ev_kernel[slot], 0));
      CK(cudaMemcpyAsync(s->h_trace[slot], s->d_trace[slot], (size_t)rows * row_floats * sizeof(float),
                         cudaMemcpyDeviceToHost, s->side));
      CK(cudaEventRecord(s->ev_copy[slot], s->side));
      pend.push_back({slot, a.step0, rows});
    }
    done += len;
    ++li;
  }
  CK(cudaEventRecord(s->ev_t1, s->stream));
  for (const Pending& p : pend) {
    int rc = drain(p);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaGetLastError());
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, s->ev_t0, s->ev_t1));
  s->last_ms = ms;
  s->last_launches = launches;
  int rc = check_device_error(s);
  if (rc) return rc;
  s->step += n_steps;
  return INFOLI_OK;
}

int infoli_sim_launch(infoli_sim* s, int n_steps) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_sim_launch");
  if (!s || n_steps < 0) return infoli__fail(INFOLI_ERR_ARG, "sim_launch: bad argument");
  CK(cudaSetDevice(s->device));
  if (int rc0 = check_table_range(s, n_steps)) return rc0;
  StepArgs a;
  fill_args(s, &a);
  a.trace_every = 0;
  a.trace_mask = 0;
  a.trace_nq = 0;
  a.trace = nullptr;
  int done = 0;
  while (done < n_steps) {
    const int len = std::min(kMaxStepsPerLaunch, n_steps - done);
    a.step0 = s->step + done;
    a.n_steps = len;
    a.stim_table = table_at(s, a.step0);
    CK(cudaMemsetAsync(s->d_bar, 0, sizeof(unsigned), s->stream));
    if (s->plan.shape.stamped) {
      CK(cudaMemsetAsync(s->d_vll[0], 0xff, (size_t)s->n_pad * sizeof(unsigned long long), s->stream));
      CK(cudaMemsetAsync(s->d_vll[1], 0xff, (size_t)s->n_pad * sizeof(unsigned long long), s->stream));
    }
    CK(launch_step_kernel(a, s->plan.grid, s->plan.threads, s->stream));
    done += len;
  }
  CK(cudaEventRecord(s->ev_t1, s->stream));
  s->step += n_steps;
  s->async_pending = 1;
  return INFOLI_OK;
}

int infoli_sim_query(infoli_sim* s) {
  infoli__clear_error();
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  if (!s->async_pending) return 1;
  CK(cudaSetDevice(s->device));
  const cudaError_t e = cudaEventQuery(s->ev_t1);
  if (e == cudaErrorNotReady) return 0;
  CK(e);
  s->async_pending = 0;
  const int rc = check_device_error(s);
  return rc ? rc : 1;
}

int infoli_sim_sync(infoli_sim* s) {
  infoli__clear_error();
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  if (!s->async_pending) return INFOLI_OK;
  s->async_pending = 0;
  return check_device_error(s);
}

namespace {
struct IntoCtx {
  float* out;
  int64_t cap;
  int n;
  int nq;
  int what;
  int rows;
  int last_step;
  int overflow;
};
void into_cb(void* user, int step, int what, const float* values, int n) {
  IntoCtx* c = (IntoCtx*)user;
  if (step != c->last_step) {
    c->last_step = step;
    c->rows++;
  }
  int qi = 0;
  for (int bit : {INFOLI_TRACE_AXON, INFOLI_TRACE_SOMA, INFOLI_TRACE_DEND}) {
    if (!(c->what & bit)) continue;
    if (bit == what) break;
    ++qi;
  }
  const int64_t off = ((int64_t)(c->rows - 1) * c->nq + qi) * n;
  if (off + n > c->cap) {
    c->overflow = 1;
    return;
  }
  std::memcpy(c->out + off, values, sizeof(float) * n);
}
}  // namespace

int infoli_sim_run_into(infoli_sim* s, int n_steps, int trace_every, int trace_what, float* out,
                        int64_t out_capacity_floats, int* rows_out) {
  infoli__clear_error();
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  if (trace_every <= 0) {
    int rc = infoli_sim_run(s, n_steps, 0, 0, nullptr, nullptr);
    if (rows_out) *rows_out = 0;
    return rc;
  }
  if (!out) return infoli__fail(INFOLI_ERR_ARG, "run_into: out is NULL");
  IntoCtx c{out, out_capacity_floats, s->n, nq_of(trace_what), trace_what, 0, -1, 0};
  int rc = infoli_sim_run(s, n_steps, trace_every, trace_what, into_cb, &c);
  if (rows_out) *rows_out = c.rows;
  if (rc) return rc;
  if (c.overflow) return infoli__fail(INFOLI_ERR_CAPACITY, "run_into: output buffer too small");
  return INFOLI_OK;
}

int infoli_sim_get_state(infoli_sim* s, float* out) {
  infoli__clear_error();
  if (!s || !out) return infoli__fail(INFOLI_ERR_ARG, "get_state: bad argument");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  // gather on the device into the ABI layout, then one device->host copy
  const int n = s->n;
  const long long total = (long long)INFOLI_NSTATE * n;
  if (int rc = state_io_buffer(s)) return rc;
  state_gather_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s->stream>>>(
      s->d_io, n, (long long)s->n_pad, state_map(), s->d_st, s->d_ca, s->d_vd[s->step & 1]);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, s->d_io, (size_t)total * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return INFOLI_OK;
}

int infoli_sim_set_state(infoli_sim* s, const float* in) {
  infoli__clear_error();
  if (!s || !in) return infoli__fail(INFOLI_ERR_ARG, "set_state: bad argument");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  return upload_state(s, in);
}

int infoli_sim_step(infoli_sim* s, int* step_out) {
  if (!s || !step_out) return infoli__fail(INFOLI_ERR_ARG, "sim_step: bad argument");
  *step_out = s->step;
  return INFOLI_OK;
}

int infoli_sim_last_run_stats(infoli_sim* s, float* device_ms, int* launches) {
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  if (device_ms) *device_ms = s->last_ms;
  if (launches) *launches = s->last_launches;
  return INFOLI_OK;
}

int infoli_sim_set_profiling(infoli_sim* s, int on) {
  infoli__clear_error();
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  if (!on) {
    if (s->d_prof) cudaFreeAsync(s->d_prof, s->stream);
    s->d_prof = nullptr;
    return INFOLI_OK;
  }
  const size_t bytes = (size_t)s->plan.grid * kProfSlots * sizeof(unsigned long long);
  if (!s->d_prof) CK(pool_alloc(&s->d_prof, bytes, s->device, s->stream));
  CK(cudaMemsetAsync(s->d_prof, 0, bytes, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return INFOLI_OK;
}

int infoli_sim_get_profile(infoli_sim* s, double mean_ns[5], double max_ns[5]) {
  infoli__clear_error();
  if (!s || !s->d_prof) return infoli__fail(INFOLI_ERR_STATE, "profiling is not enabled");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  std::vector<unsigned long long> h((size_t)s->plan.grid * kProfSlots);
  CK(cudaMemcpy(h.data(), s->d_prof, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  const int slot_of[5] = {PROF_STAGE, PROF_COUPLE, PROF_UPDATE, PROF_BARRIER, PROF_UNITS};
  // cycles -> ns with the clock seen over the launches (global timer / SM cycles)
  double span_ns = 0, span_cy = 0;
  for (int b = 0; b < s->plan.grid; ++b) {
    span_ns += (double)h[(size_t)b * kProfSlots + PROF_SPAN_NS];
    span_cy += (double)h[(size_t)b * kProfSlots + PROF_SPAN_CYCLES];
  }
  const double ns_per_cycle = span_cy > 0 ? span_ns / span_cy : 0.0;
  for (int k = 0; k < 5; ++k) {
    double sum = 0, mx = 0;
    for (int b = 0; b < s->plan.grid; ++b) {
      const unsigned long long steps = h[(size_t)b * kProfSlots + PROF_STEPS];
      const double v =
          steps ? ns_per_cycle * (double)h[(size_t)b * kProfSlots + slot_of[k]] / (double)steps : 0.0;
      sum += v;
      mx = std::max(mx, v);
    }
    if (mean_ns) mean_ns[k] = sum / std::max(1, s->plan.grid);
    if (max_ns) max_ns[k] = mx;
  }
  return INFOLI_OK;
}

int infoli_sim_plan_info(infoli_sim* s, int* grid, int* threads, int* tiles, int* chunks, int64_t* smem_bytes) {
  if (!s) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  if (grid) *grid = s->plan.grid;
  if (threads) *threads = s->plan.threads;
  if (tiles) *tiles = (int)s->plan.tiles.size();
  if (chunks) *chunks = (int)s->plan.chunks.size();
  if (smem_bytes) *smem_bytes = (int64_t)s->plan.smem_bytes;
  return INFOLI_OK;
}

}  // extern "C"
