// Allocation-free entry point: infoli_run_noalloc.
//
// Some callers cannot allocate device memory while they drive the
// simulation: hosts that reserved a fixed device-memory arena at start-up and
// hand the library pieces of it (an allocation outside the arena can fail or
// break the budget), foreign-language bindings whose runtime's allocator owns
// every device buffer (memory taken behind its back escapes its accounting),
// and loops running beside other GPU work that cannot take the device-wide
// synchronisation cudaFree (and often cudaMalloc) implies.  For them this file
// offers one entry point that allocates nothing: the caller passes the
// network, the state and the trace buffer in device memory, and the only
// scratch the kernel needs -- the V_dend double buffer shared between CTAs,
// the grid-barrier counter and the error word -- lives in one file-scope
// static __device__ array of fixed size (kNoAllocMaxCells cells, about 0.5
// MiB), which every GPU that loads the library keeps until the process exits.
//
// The kernel is a variant of the persistent step kernel: one thread per cell
// runs the coupling sum straight from the CSR lists (gathering V_dend from
// the shared scratch buffer) and the fused compartment update with
// register-resident state, with one grid barrier per step.  The barrier
// counter is 64-bit, so one call may run any number of steps without it
// wrapping.  Malformed topology (a sender id outside [0, n), a NULL column
// array with edges, a decreasing or negative row_ptr) is recorded in the
// error word and the bad read is skipped, so it never reads outside the
// caller's buffers through a bad index; row_ptr[n] itself cannot be checked
// against the length of the caller's arrays and is the caller's contract.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/infoli_gpu.h"
#include "infoli_cell.cuh"
#include "infoli_internal.h"
#include "infoli_ptx.cuh"

namespace infoli {
namespace {

constexpr int kNoAllocMaxCells = 65536;  // largest network the static scratch holds
constexpr int kNoAllocBlock = 512;
constexpr int kMaxDevices = 64;

// Scratch layout: [0, 256) 64-bit barrier counter at 0 + error word at 64
// (zeroed before every launch); [256, ...) V_dend double buffer,
// 2 x kNoAllocMaxCells floats.
constexpr int kErrBarrier = 1, kErrSender = 2, kErrRowPtr = 3;
constexpr size_t kCtlBytes = 256;
constexpr size_t kScratchBytes = kCtlBytes + 2 * sizeof(float) * (size_t)kNoAllocMaxCells;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr float kNegLog2eOver100 = -0.014426950408889634f;  // -log2(e)/100

struct NoAllocArgs {
  ModelParams P;
  int n, step0, n_steps;
  const int64_t* row_ptr;
  const int32_t* col;
  const float* g;
  float g_uniform;
  int pulse_start, pulse_end;
  float pulse_amp;
  float* state;        // INFOLI_NSTATE x n, reference order (V_dend first)
  float* trace_axon;   // n_steps x n, or null
  unsigned char* scratch;  // device address of g_noalloc_scratch
  unsigned long long timeout_ns;
};

__device__ __forceinline__ bool noalloc_barrier(const NoAllocArgs& a, unsigned long long* bar, int* err,
                                                unsigned long long target) {
  __shared__ int s_abort;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_abort = 0;
    __threadfence();
    red_release_gpu_add_u64(bar, 1ull);
    const uint64_t t0 = globaltimer_ns();
    while (ld_acquire_gpu_u64(bar) < target) {
      if (ld_relaxed_gpu(err) != 0 || globaltimer_ns() - t0 > a.timeout_ns) {
        atomicCAS(err, 0, kErrBarrier);
        s_abort = 1;
        break;
      }
    }
  }
  __syncthreads();
  return s_abort == 0;
}

__global__ void __launch_bounds__(kNoAllocBlock, 1) noalloc_step_kernel(const __grid_constant__ NoAllocArgs a) {
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(a.scratch);
  int* err = reinterpret_cast<int*>(a.scratch + 64);
  float* vd[2] = {reinterpret_cast<float*>(a.scratch + kCtlBytes),
                  reinterpret_cast<float*>(a.scratch + kCtlBytes) + kNoAllocMaxCells};
  const int n = a.n;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool own = c < n;
  const size_t N = (size_t)n;

  // reference state order: V_dend, Calcium_r, Potassium_s, Hcurrent_q,
  // Ca2Plus, I_CaH, g_CaL, V_soma, Sodium_m, Sodium_h, Potassium_n,
  // Potassium_p, Potassium_x_s, Calcium_k, Calcium_l, V_axon, Sodium_m_a,
  // Sodium_h_a, Potassium_x_a
  Volts v{};
  Gates gs{};
  if (own) {
    const float* s = a.state;
    v.Vd = s[0 * N + c];
    gs.r = s[1 * N + c];
    gs.s = s[2 * N + c];
    gs.q = s[3 * N + c];
    gs.Ca = (double)s[4 * N + c];
    gs.ICaH = s[5 * N + c];
    gs.gCaL = s[6 * N + c];
    v.Vs = s[7 * N + c];
    gs.m = s[8 * N + c];
    gs.h = s[9 * N + c];
    gs.n = s[10 * N + c];
    gs.p = s[11 * N + c];
    gs.xs = s[12 * N + c];
    gs.k = s[13 * N + c];
    gs.l = s[14 * N + c];
    v.Va = s[15 * N + c];
    gs.ma = s[16 * N + c];
    gs.ha = s[17 * N + c];
    gs.xa = s[18 * N + c];
    vd[a.step0 & 1][c] = v.Vd;
  }
  unsigned long long target = gridDim.x;
  bool ok = noalloc_barrier(a, bar, err, target);
  // this thread's edge range, checked once (a bad row is recorded and skipped)
  int64_t e_begin = 0, e_end = 0;
  if (own) {
    e_begin = a.row_ptr[c];
    e_end = a.row_ptr[c + 1];
    if (e_begin < 0 || e_end < e_begin) {
      atomicCAS(err, 0, kErrRowPtr);
      e_end = e_begin;
    } else if (e_end > e_begin && a.col == nullptr) {
      atomicCAS(err, 0, kErrSender);
      e_end = e_begin;
    }
  }
  const VoltCoef vk = volt_coef(a.P);
  for (int t = 0; t < a.n_steps && ok; ++t) {
    const int step = a.step0 + t;
    if (own) {
      const float* vcur = vd[step & 1];
      float acc = 0.0f;
      for (int64_t e = e_begin; e < e_end; ++e) {
        const int s = a.col[e];
        if ((unsigned)s >= (unsigned)n) {  // malformed topology: record, never read outside the buffer
          atomicCAS(err, 0, kErrSender);
          continue;
        }
        const float V = v.Vd - __ldcg(vcur + s);  // L2: written by other CTAs this launch
        const float f = fmaf(0.8f, ex2_approx((V * V) * kNegLog2eOver100), 0.2f);
        acc += a.g ? (a.g[e] * f) * V : f * V;
      }
      const float ic = a.g ? acc : acc * a.g_uniform;
      const float iapp = (step >= a.pulse_start && step < a.pulse_end) ? a.pulse_amp : 0.0f;
      Currents cur;
      run_units(a.P, 0xffu, v, gs, cur);
      voltage_step(a.P, vk, v, cur, ic, iapp);
      vd[(step + 1) & 1][c] = v.Vd;
      if (a.trace_axon) a.trace_axon[(size_t)t * N + c] = v.Va;
    }
    target += gridDim.x;
    ok = noalloc_barrier(a, bar, err, target);
  }
  if (own) {
    float* s = a.state;
    s[0 * N + c] = v.Vd;
    s[1 * N + c] = gs.r;
    s[2 * N + c] = gs.s;
    s[3 * N + c] = gs.q;
    s[4 * N + c] = (float)gs.Ca;
    s[5 * N + c] = gs.ICaH;
    s[7 * N + c] = v.Vs;
    s[8 * N + c] = gs.m;
    s[9 * N + c] = gs.h;
    s[10 * N + c] = gs.n;
    s[11 * N + c] = gs.p;
    s[12 * N + c] = gs.xs;
    s[13 * N + c] = gs.k;
    s[14 * N + c] = gs.l;
    s[15 * N + c] = v.Va;
    s[16 * N + c] = gs.ma;
    s[17 * N + c] = gs.ha;
    s[18 * N + c] = gs.xa;
  }
}

std::mutex g_scratch_mu;
unsigned char* g_scratch_addr[kMaxDevices];

}  // namespace
}  // namespace infoli

using namespace infoli;

extern "C" int infoli_run_noalloc(const float* params, int n_cells, const int64_t* d_row_ptr, const int32_t* d_col,
                                  const float* d_g, float g_uniform, int pulse_start, int pulse_end, float pulse_amp,
                                  float* d_state, int step0, int n_steps, float* d_trace_axon, void* stream) {
  infoli__clear_error();
  if (!params || !d_row_ptr || !d_state || n_cells <= 0 || n_steps < 0 || step0 < 0)
    return infoli__fail(INFOLI_ERR_ARG, "run_noalloc: bad argument");
  if ((long long)step0 + (long long)n_steps > (long long)INT_MAX)
    return infoli__fail(INFOLI_ERR_ARG, "run_noalloc: step0 + n_steps exceeds INT_MAX");
  if (n_cells > kNoAllocMaxCells)
    return infoli__fail(INFOLI_ERR_CAPACITY,
                        "run_noalloc: %d cells exceed the static scratch limit of %d cells; use infoli_sim_create",
                        n_cells, kNoAllocMaxCells);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return infoli__fail(INFOLI_ERR_ARG, "run_noalloc: device %d out of range", dev);
  unsigned char* scratch = nullptr;
  {
    // once per device, with that device current: the symbol's device address
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  int nsm = 0;
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess)
    return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: cudaDeviceGetAttribute: %s", cudaGetErrorString(e));
  const int grid = (n_cells + kNoAllocBlock - 1) / kNoAllocBlock;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, noalloc_step_kernel, kNoAllocBlock, 0);
  if (e != cudaSuccess)
    return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: occupancy query: %s", cudaGetErrorString(e));
  if (grid > per_sm * nsm)
    return infoli__fail(INFOLI_ERR_CAPACITY, "run_noalloc: %d CTAs cannot be co-resident (%d allowed)", grid,
                        per_sm * nsm);
  NoAllocArgs a{};
  static_assert(sizeof(ModelParams) == INFOLI_NPARAM * sizeof(float), "param layout");
  memcpy(&a.P, params, sizeof(ModelParams));
  a.n = n_cells;
  a.step0 = step0;
  a.n_steps = n_steps;
  a.row_ptr = d_row_ptr;
  a.col = d_col;
  a.g = d_g;
  a.g_uniform = g_uniform;
  a.pulse_start = pulse_start;
  a.pulse_end = pulse_end;
  a.pulse_amp = pulse_amp;
  a.state = d_state;
  a.trace_axon = d_trace_axon;
  a.scratch = scratch;
  a.timeout_ns = infoli__wait_timeout_ns();
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the barrier counter and the error word must start at zero
  e = cudaMemsetAsync(scratch, 0, kCtlBytes, s);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: cudaMemsetAsync: %s", cudaGetErrorString(e));
  void* args[] = {&a};
  e = cudaLaunchCooperativeKernel((const void*)noalloc_step_kernel, dim3(grid), dim3(kNoAllocBlock), args, 0, s);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: launch: %s", cudaGetErrorString(e));
  // the error word comes back on the caller's stream: a plain cudaMemcpy would
  // go to the legacy default stream and wait for every blocking stream
  int err = 0;
  e = cudaMemcpyAsync(&err, scratch + 64, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: %s", cudaGetErrorString(e));
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return infoli__fail(INFOLI_ERR_CUDA, "run_noalloc: %s", cudaGetErrorString(e));
  if (err == kErrSender)
    return infoli__fail(INFOLI_ERR_ARG, "run_noalloc: a sender id is outside [0, n_cells) (or d_col is NULL)");
  if (err == kErrRowPtr) return infoli__fail(INFOLI_ERR_ARG, "run_noalloc: d_row_ptr is negative or decreasing");
  if (err) return infoli__fail(INFOLI_ERR_TIMEOUT, "run_noalloc: grid barrier wait gave up");
  return INFOLI_OK;
}
