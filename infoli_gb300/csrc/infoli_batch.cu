// Batched simulation of many independent networks in one captured graph.
//
// Each network's cells are split over the CTAs of ONE thread-block cluster
// (up to 8 CTAs of 1024 threads; one thread per cell, state in registers).
// Every CTA keeps the whole network's V_dend, double-buffered, in its shared
// memory; a new V_dend is written to the CTA's own copy and, through
// distributed shared memory, to the copies of the network's other CTAs, and
// the cluster's hardware barrier separates the steps.  No grid-wide
// synchronisation: every cluster runs its network independently.  Networks
// needing the same number of CTAs form one launch with that cluster size, so
// clusters have no idle CTA; the launches run concurrently.
//
// Coupling is read from per-network adjacency bitmasks with one conductance
// per network (the reference's uniform CONDUCTANCE, src/openmp/infoli.c:320):
// a receiver walks the set bits of its row (src/openmp/infoli.c:512-518 for
// the arithmetic).  Rows are stored word-major so consecutive receivers read
// consecutive words; a network whose rows fit keeps them in shared memory for
// the launch, otherwise they are streamed from global memory every step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/infoli_gpu.h"
#include "infoli_cell.cuh"
#include "infoli_internal.h"
#include "infoli_ptx.cuh"

namespace infoli {
namespace {

constexpr float kNegLog2eOver100 = -0.014426950408889634f;  // -log2(e)/100

}  // namespace
}  // namespace infoli

#include "infoli_lane.h"

namespace infoli {
namespace {

struct BatchArgs {
  ModelParams P;
  const BatchCta* cta;
  int vcap;          // floats per V buffer in shared memory
  int res_words;     // shared words for resident rows (per CTA)
  const int* step;   // current step index of the batch (device), for CTAs whose step0 < 0
  int n_steps;       // steps of the launch, for CTAs whose n_steps < 0
  unsigned long long* cta_ns;  // [2 * grid]: globaltimer at start and end of every CTA
};

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Store a float into the shared memory of CTA `peer` of this cluster at the
// address that `local` has in this CTA.
// The V_dend buffers hold V * kVScale (kVScale^2 = log2(e) / 100), so a
// coupling term's exponent is -(dV')^2 with dV' = kVScale dV: one multiply
// less per edge; the sums are scaled back once per receiver.
constexpr float kVScale = 0.12011224087864497f;
constexpr float kInvVScale = 8.325546111576978f;

__device__ __forceinline__ void st_peer(float* local, unsigned peer, float v) {
  const unsigned la = smem_u32(local);
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(peer));
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra), "f"(v) : "memory");
}

// Gap-junction currents of a warp's 32 receivers from their bitmask rows,
// one 32-sender column of the rows at a time.  Words are stored
// most-significant-bit first (bit 31 of word w = sender 32 w), so a count of
// leading zeros is the sender's offset within the column.  For each column
// the warp runs as many iterations as the fullest word of its lanes has bits
// (a warp-wide max of the popcounts); an iteration takes the next set bit of
// every lane's word and reads that sender's V_dend.  All lanes read from the
// same 32 consecutive floats, so the reads never conflict on a shared-memory
// bank, and the loop has no divergent branch.  A lane whose word is used up
// reads a float past the column (inside the V_dend buffer's 32-float tail
// pad) and adds nothing.  Senders are visited in ascending order (the
// reference's order); the terms of a column are summed in FP32 and, with
// KAHAN, the column sums are added with Kahan compensation.  Lanes without a
// receiver pass own == false.
//   RES: words in shared memory at byte address wsm + 4 * BLOCK * w;
//   else words in global memory at gw[w * stride].
// Lockstep iterations per trip of the column walk.
#ifndef INFOLI_BATCH_UNROLL
#define INFOLI_BATCH_UNROLL 2
#endif

// One lockstep iteration: the lane's next set bit of x (leading zeros; 32
// once x is used up, which reads a pad float and adds nothing), that
// sender's V_dend x kVScale, its term added to col.
__device__ __forceinline__ void batch_take(uint32_t& x, uint32_t vcol, float vc, float& col) {
  const int c = __clz(x);
  const bool live = x != 0u;
  x &= __funnelshift_rc(0x7fffffffu, 0u, (unsigned)c);
  const float V = vc - ld_shared_f32(vcol + 4u * (uint32_t)c);  // scaled by kVScale
  const float f = fmaf(0.8f, ex2_approx(-(V * V)), 0.2f);
  if (live) col = fmaf(f, V, col);
}

template <bool KAHAN, bool RES>
__device__ __forceinline__ float couple_warp(bool own, uint32_t wsm, uint32_t wstride_b, const uint32_t* gw,
                                            uint32_t stride, int wpr, uint32_t vbase, float vc) {
  float acc = 0.0f, cmp = 0.0f;
  uint32_t nx = 0u, nnx = 0u;
  if (own) {
    if (RES) {
      ld_shared_if(nx, wsm, true);
      ld_shared_if(nnx, wsm + wstride_b, wpr > 1);
    } else {
      nx = __ldg(gw);
      if (wpr > 1) nnx = __ldg(gw + stride);
    }
  }
  for (int w = 0; w < wpr; ++w) {
    uint32_t x = nx;
    nx = nnx;
    // words w + 2 are loaded two columns ahead (rows end with two zero words)
    if (RES)
      ld_shared_if(nnx, wsm + (uint32_t)(w + 2) * wstride_b, own);
    else
      ld_global_if(nnx, gw + (size_t)(w + 2) * stride, own);
    const int m = (int)__reduce_max_sync(0xffffffffu, (unsigned)__popc(x));
    const uint32_t vcol = vbase + 128u * (uint32_t)w;
    float col = 0.0f;  // this column's terms (at most 32)
    // INFOLI_BATCH_UNROLL iterations per trip, then the rest one at a time:
    // the same terms in the same order either way
    int k = 0;
    for (; k + INFOLI_BATCH_UNROLL <= m; k += INFOLI_BATCH_UNROLL) {
#pragma unroll
      for (int u = 0; u < INFOLI_BATCH_UNROLL; ++u) batch_take(x, vcol, vc, col);
    }
#pragma unroll 1
    for (; k < m; ++k) batch_take(x, vcol, vc, col);
    if (KAHAN) {
      // compensated sum over the column sums
      const float y = col - cmp;
      const float s = acc + y;
      cmp = (s - acc) - y;
      acc = s;
    } else {
      acc += col;
    }
  }
  return acc;
}

// BLOCK threads per CTA and 1024 / BLOCK CTAs per SM (64 registers per thread
// either way).  Only the CTA record's hot fields are held in registers; the
// state pointers, stride and pulse are read from the record where they are
// used (the cluster barriers' memory clobbers keep the compiler from holding
// them across the step loop).
template <int BLOCK, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* vbuf = reinterpret_cast<float*>(smem_raw);              // [2][vcap]
  uint32_t* sbits = reinterpret_cast<uint32_t*>(vbuf + 2 * a.vcap);  // [wpr + 2][BLOCK] if resident
  const unsigned long long t_start = globaltimer_ns();
  const BatchCta* wp = a.cta + blockIdx.x;
  const int net = wp->net, ncell = wp->ncell, n = wp->n, wpr = wp->wpr;
  const int ncta = wp->ncta, rank0 = wp->rank0;
  const bool resident = wp->resident != 0, cl_sync = wp->cl_sync != 0;
  const int tid = threadIdx.x;
  const unsigned me = cluster_rank();
  const bool own = net >= 0 && tid < ncell;
  const int r = wp->cbeg + tid;
  const int step0 = wp->step0 >= 0 ? wp->step0 : *a.step;
  const int n_steps = wp->n_steps >= 0 ? wp->n_steps : a.n_steps;  // the same in every CTA of a cluster
  const uint32_t* gbits = wp->bits;

  Volts v{};
  Gates gs{};
  if (own) {
    const long long T = wp->T, gc = wp->cell_base + r;
    const float* s = wp->st;
    v.Vd = s[0 * T + gc];
    gs.r = s[1 * T + gc];
    gs.s = s[2 * T + gc];
    gs.q = s[3 * T + gc];
    gs.Ca = wp->ca[gc];
    gs.ICaH = s[5 * T + gc];
    gs.gCaL = s[6 * T + gc];
    v.Vs = s[7 * T + gc];
    gs.m = s[8 * T + gc];
    gs.h = s[9 * T + gc];
    gs.n = s[10 * T + gc];
    gs.p = s[11 * T + gc];
    gs.xs = s[12 * T + gc];
    gs.k = s[13 * T + gc];
    gs.l = s[14 * T + gc];
    v.Va = s[15 * T + gc];
    gs.ma = s[16 * T + gc];
    gs.ha = s[17 * T + gc];
    gs.xa = s[18 * T + gc];
  }
  if (net >= 0 && resident) {
    for (int i = tid; i < (wpr + 2) * BLOCK; i += BLOCK) {
      const int ww = i / BLOCK, rr = i % BLOCK;
      sbits[i] = rr < ncell ? gbits[(long long)ww * n + wp->cbeg + rr] : 0u;
    }
  }
  cluster_sync_all();  // every CTA of the cluster is running before peers write into it
  if (own) {
    vbuf[r] = v.Vd * kVScale;
    for (int p = 0; p < ncta; ++p)
      if (rank0 + p != (int)me) st_peer(vbuf + r, (unsigned)(rank0 + p), v.Vd * kVScale);
  }
  cluster_sync_all();

  const VoltCoef vk = volt_coef(a.P);
  for (int t = 0; t < n_steps; ++t) {
    const int step = step0 + t;
    const float* vcur = vbuf + (t & 1) * a.vcap;
    float* vnxt = vbuf + ((t + 1) & 1) * a.vcap;
    // ---- coupling: the set bits of the rows (whole warps, owned or not)
    float sum = 0.0f;
    if (net >= 0 && (tid & ~31) < ncell) {
      const uint32_t vbase = smem_u32(vcur);
      const float vcs = v.Vd * kVScale;
      sum = resident ? couple_warp<KAHAN, true>(own, smem_u32(sbits + tid), 4u * BLOCK, nullptr, 0u, wpr, vbase, vcs)
                     : couple_warp<KAHAN, false>(own, 0u, 0u, gbits + r, (uint32_t)n, wpr, vbase, vcs);
    }
    if (own) {
      const float ic = sum * (wp->g * kInvVScale);
      const float iapp = (step >= wp->pulse_start && step < wp->pulse_end) ? wp->pulse_amp : 0.0f;
      // ---- fused compartment update
      Currents cur;
      run_units(a.P, 0xffu, v, gs, cur);
      voltage_step(a.P, vk, v, cur, ic, iapp);
      const float vds = v.Vd * kVScale;
      vnxt[r] = vds;
      for (int p = 0; p < ncta; ++p)
        if (rank0 + p != (int)me) st_peer(vnxt + r, (unsigned)(rank0 + p), vds);
    }
    if (cl_sync)
      cluster_sync_all();
    else
      __syncthreads();
  }

  if (own) {
    const long long T = wp->T, gc = wp->cell_base + r;
    float* s = wp->st;
    s[0 * T + gc] = v.Vd;
    s[1 * T + gc] = gs.r;
    s[2 * T + gc] = gs.s;
    s[3 * T + gc] = gs.q;
    wp->ca[gc] = gs.Ca;
    s[5 * T + gc] = gs.ICaH;
    s[7 * T + gc] = v.Vs;
    s[8 * T + gc] = gs.m;
    s[9 * T + gc] = gs.h;
    s[10 * T + gc] = gs.n;
    s[11 * T + gc] = gs.p;
    s[12 * T + gc] = gs.xs;
    s[13 * T + gc] = gs.k;
    s[14 * T + gc] = gs.l;
    s[15 * T + gc] = v.Va;
    s[16 * T + gc] = gs.ma;
    s[17 * T + gc] = gs.ha;
    s[18 * T + gc] = gs.xa;
  }
  if (tid == 0) {
    a.cta_ns[2 * blockIdx.x] = t_start;
    a.cta_ns[2 * blockIdx.x + 1] = globaltimer_ns();
  }
}

__global__ void batch_advance(int* step, int n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += n;
}

}  // namespace
}  // namespace infoli

using namespace infoli;

namespace {

// Networks that need the same number of CTAs form a group; a group is one
// kernel launch whose clusters have exactly that many CTAs, one network per
// cluster, so no cluster has an idle CTA.  The groups run concurrently (one
// stream each, forked and joined inside the captured graph), the groups of
// the largest networks first and at the highest priority.
struct BatchGroup {
  int cs = 1;             // CTAs per cluster = CTAs per network
  int cta_off = 0, grid = 0;
  int vcap = 0, res_words = 0;
  size_t smem = 0;
  int max_active = 0;     // clusters of this group the device runs at once
  int priority = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

}  // namespace

struct infoli_batch {
  int device = 0;
  int n_nets = 0;
  long long total = 0;
  ModelParams P{};
  int kahan = 0;
  int block = 1024;
  std::vector<BatchGroup> groups;
  std::vector<BatchCta> cta;
  std::vector<long long> cell_base;
  BatchCta* d_cta = nullptr;
  uint32_t* d_bits = nullptr;
  float* d_st = nullptr;
  double* d_ca = nullptr;
  int* d_step = nullptr;
  unsigned long long* d_cta_ns = nullptr;
  int pulse_start = 20000, pulse_end = 20499;
  float pulse_amp = 6.0f;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_steps = -1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0;
};

namespace {

#define BK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return infoli__fail(INFOLI_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                          __LINE__);                                                               \
  } while (0)

uint32_t reverse_bits(uint32_t x) {
  x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
  x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
  x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
  x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
  return (x >> 16) | (x << 16);
}

void batch_release(infoli_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (void* p : {(void*)b->d_cta, (void*)b->d_bits, (void*)b->d_st, (void*)b->d_ca, (void*)b->d_step,
                  (void*)b->d_cta_ns})
    if (p) cudaFree(p);
  for (BatchGroup& g : b->groups) {
    if (g.done) cudaEventDestroy(g.done);
    if (g.stream) cudaStreamDestroy(g.stream);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const void* kernel_ptr(int block, bool kahan) {
  if (block == 512) return kahan ? (const void*)batch_kernel<512, true> : (const void*)batch_kernel<512, false>;
  return kahan ? (const void*)batch_kernel<1024, true> : (const void*)batch_kernel<1024, false>;
}

// Kernel attributes are set before any capture (cudaFuncSetAttribute is not a
// stream operation).
cudaError_t set_attrs(int block, size_t smem, int cluster) {
  for (int k = 0; k < 2; ++k) {
    const void* fn = kernel_ptr(block, k == 1);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && cluster > 8) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void fill_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* at, int grid, int block, int cluster, size_t smem,
                 int priority, cudaStream_t s) {
  cfg = cudaLaunchConfig_t{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributePriority;
  at[1].val.priority = priority;
  cfg.attrs = at;
  cfg.numAttrs = 2;
}

int max_clusters(int block, int cluster, size_t smem) {
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[2];
  fill_config(cfg, at, cluster, block, cluster, smem, 0, nullptr);
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel_ptr(block, false), &cfg) != cudaSuccess) return 0;
  return n;
}

cudaError_t launch_group(const infoli_batch* b, const BatchGroup& g, BatchArgs a) {
  a.cta += g.cta_off;
  a.cta_ns += 2 * (size_t)g.cta_off;
  a.vcap = g.vcap;
  a.res_words = g.res_words;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[2];
  fill_config(cfg, at, g.grid, b->block, g.cs, g.smem, g.priority, g.stream);
  if (b->block == 512)
    return b->kahan ? cudaLaunchKernelEx(&cfg, batch_kernel<512, true>, a)
                    : cudaLaunchKernelEx(&cfg, batch_kernel<512, false>, a);
  return b->kahan ? cudaLaunchKernelEx(&cfg, batch_kernel<1024, true>, a)
                  : cudaLaunchKernelEx(&cfg, batch_kernel<1024, false>, a);
}

}  // namespace

extern "C" int infoli_batch_create(const infoli_batch_desc* d, infoli_batch** out) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_batch_create");
  if (!d || !out || d->n_nets <= 0 || !d->n_cells || !d->params || !d->bits || !d->g ||
      (!d->init_state && !d->init_values))
    return infoli__fail(INFOLI_ERR_ARG, "batch_create: bad argument");
  *out = nullptr;
  infoli_batch* b = new infoli_batch();
  auto fail = [&](int rc) {
    batch_release(b);
    return rc;
  };
  b->device = d->device;
  b->n_nets = d->n_nets;
  b->kahan = (d->flags & INFOLI_F_KAHAN) ? 1 : 0;
  std::memcpy(&b->P, d->params, sizeof(ModelParams));
  if (d->block != 0 && d->block != 512 && d->block != 1024)
    return fail(infoli__fail(INFOLI_ERR_ARG, "batch_create: block %d (0, 512 or 1024)", d->block));
  if (d->residency < INFOLI_RES_FIT || d->residency > INFOLI_RES_NONE)
    return fail(infoli__fail(INFOLI_ERR_ARG, "batch_create: residency %d (0, 1 or 2)", d->residency));
  if (cudaSetDevice(b->device) != cudaSuccess) return fail(infoli__fail(INFOLI_ERR_CUDA, "cudaSetDevice failed"));
  if (d->block != 0) {
    b->block = d->block;
  } else {
    const char* shape_env = getenv("INFOLI_BATCH_SHAPE");
    b->block = (shape_env && atoi(shape_env) == 512) ? 512 : 1024;
  }
  const int max_cs = b->block == 1024 ? 8 : 16;
  b->cell_base.resize(d->n_nets);
  long long bits_total = 0, in_total = 0;
  std::vector<long long> bits_base(d->n_nets), in_base(d->n_nets);
  for (int i = 0; i < d->n_nets; ++i) {
    const int n = d->n_cells[i];
    if (n <= 0) return fail(infoli__fail(INFOLI_ERR_ARG, "batch_create: network %d has no cells", i));
    if ((n + b->block - 1) / b->block > max_cs)
      return fail(infoli__fail(INFOLI_ERR_CAPACITY, "batch_create: network %d has %d cells (at most %d)", i, n,
                               b->block * max_cs));
    b->cell_base[i] = b->total;
    b->total += n;
    in_base[i] = in_total;
    in_total += (long long)n * ((n + 31) / 32);
    bits_base[i] = bits_total;
    bits_total += (long long)n * ((n + 31) / 32 + 2);
  }
  // time per step of a network ~ its mean row weight (set bits per receiver)
  // plus a constant for the cell update: heavy networks are launched first
  std::vector<double> weight(d->n_nets);
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < d->n_nets; ++i) {
    const int n = d->n_cells[i], wpr = (n + 31) / 32;
    const uint32_t* src = d->bits + in_base[i];
    long long ones = 0;
    for (long long k = 0; k < (long long)n * wpr; ++k) ones += __builtin_popcount(src[k]);
    weight[i] = (double)ones / n + 64.0;
  }
  int smem_optin = 0, smem_sm = 0, prio_lo = 0, prio_hi = 0;
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, b->device);
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  const size_t budget = (size_t)smem_optin - 1024;
  // shared memory a group may spend on resident rows: all of a CTA's budget
  // (FIT), what keeps 2048 / block CTAs on an SM (OCC; the runtime reserves
  // 1 KB per CTA), or nothing (NONE)
  const int ctas_per_sm = 2048 / b->block;
  const size_t occ_budget = std::min(budget, (size_t)smem_sm / (size_t)ctas_per_sm - 1024);
  const size_t res_budget = d->residency == INFOLI_RES_NONE ? 0
                            : d->residency == INFOLI_RES_OCC ? occ_budget : budget;
  for (int cs = max_cs; cs >= 1; --cs) {
    std::vector<int> nets;
    for (int i = 0; i < d->n_nets; ++i)
      if ((d->n_cells[i] + b->block - 1) / b->block == cs) nets.push_back(i);
    if (nets.empty()) continue;
    std::stable_sort(nets.begin(), nets.end(), [&](int x, int y) { return weight[x] > weight[y]; });
    BatchGroup g;
    g.cs = cs;
    g.cta_off = (int)b->cta.size();
    int nmax = 0;
    for (int i : nets) nmax = std::max(nmax, d->n_cells[i]);
    g.vcap = ((nmax + 31) / 32) * 32 + 32;  // + the 32-float pad read by finished lanes
    const size_t vbytes = 2 * sizeof(float) * (size_t)g.vcap;
    int res_rows = 0;  // words per resident row (wpr + 2), max over resident networks
    for (int i : nets) {
      const int wr = (d->n_cells[i] + 31) / 32 + 2;
      if (vbytes + sizeof(uint32_t) * (size_t)wr * b->block <= res_budget) res_rows = std::max(res_rows, wr);
    }
    g.res_words = res_rows * b->block;
    g.smem = vbytes + sizeof(uint32_t) * (size_t)g.res_words;
    if (g.smem > budget)
      return fail(infoli__fail(INFOLI_ERR_CAPACITY, "batch_create: %zu bytes of shared memory needed", g.smem));
    if (set_attrs(b->block, budget, max_cs) != cudaSuccess || (g.max_active = max_clusters(b->block, cs, g.smem)) <= 0)
      return fail(infoli__fail(INFOLI_ERR_CAPACITY, "batch_create: clusters of %d CTAs of %d threads cannot run",
                               cs, b->block));
    // greatest priority for the largest networks
    g.priority = std::max(prio_hi, std::min(prio_lo, prio_hi + (max_cs - cs) * (prio_lo - prio_hi) / max_cs));
    for (int i : nets) {
      const int n = d->n_cells[i];
      const int per = (n + cs - 1) / cs;
      for (int k = 0; k < cs; ++k) {
        BatchCta w{};
        w.net = i;
        w.rank = k;
        w.ncta = cs;
        w.rank0 = 0;
        w.cbeg = std::min(n, k * per);
        w.ncell = std::min(n, (k + 1) * per) - w.cbeg;
        w.n = n;
        w.wpr = (n + 31) / 32;
        w.cell_base = b->cell_base[i];
        w.T = 0;  // device pointers and the stride are filled in after the allocation
        w.g = d->g[i];
        w.n_steps = -1;
        w.step0 = -1;
        w.pulse_start = b->pulse_start;
        w.pulse_end = b->pulse_end;
        w.pulse_amp = b->pulse_amp;
        w.resident = (w.wpr + 2) * b->block <= g.res_words ? 1 : 0;
        w.cl_sync = cs > 1 ? 1 : 0;
        b->cta.push_back(w);
      }
    }
    g.grid = (int)b->cta.size() - g.cta_off;
    b->groups.push_back(g);
  }

  // Device bitmasks, word-major (word w of receiver r at base + w * n + r),
  // most-significant bit first, two zero words after every row.
  std::vector<uint32_t> tb((size_t)bits_total, 0u);
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < d->n_nets; ++i) {
    const int n = d->n_cells[i], wpr = (n + 31) / 32;
    const uint32_t* src = d->bits + in_base[i];
    uint32_t* dst = tb.data() + bits_base[i];
    for (int r = 0; r < n; ++r)
      for (int wd = 0; wd < wpr; ++wd) {
        uint32_t x = src[(size_t)r * wpr + wd];
        if (wd == r / 32) x &= ~(1u << (r % 32));  // no self-coupling
        if (wd == wpr - 1 && n % 32) x &= (1u << (n % 32)) - 1u;
        dst[(size_t)wd * n + r] = reverse_bits(x);
      }
  }
  std::vector<float> st((size_t)INFOLI_NSTATE * b->total);
  if (d->init_state) {
    std::memcpy(st.data(), d->init_state, st.size() * sizeof(float));
  } else {
    for (int k = 0; k < INFOLI_NSTATE; ++k)
      std::fill(st.begin() + (size_t)k * b->total, st.begin() + (size_t)(k + 1) * b->total, d->init_values[k]);
  }
  std::vector<double> ca(st.begin() + 4 * b->total, st.begin() + 5 * b->total);
  if (cudaMalloc((void**)&b->d_cta, sizeof(BatchCta) * b->cta.size()) != cudaSuccess ||
      cudaMalloc((void**)&b->d_bits, sizeof(uint32_t) * std::max<size_t>(1, tb.size())) != cudaSuccess ||
      cudaMalloc((void**)&b->d_st, sizeof(float) * st.size()) != cudaSuccess ||
      cudaMalloc((void**)&b->d_ca, sizeof(double) * b->total) != cudaSuccess ||
      cudaMalloc((void**)&b->d_step, sizeof(int)) != cudaSuccess ||
      cudaMalloc((void**)&b->d_cta_ns, sizeof(unsigned long long) * 2 * b->cta.size()) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_NOMEM, "batch_create: device allocation failed"));
  for (BatchCta& w : b->cta) {
    w.st = b->d_st;
    w.ca = b->d_ca;
    w.bits = b->d_bits + bits_base[w.net];
    w.T = b->total;
  }
  if (cudaMemcpy(b->d_cta, b->cta.data(), sizeof(BatchCta) * b->cta.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_bits, tb.data(), sizeof(uint32_t) * tb.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_st, st.data(), sizeof(float) * st.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->d_ca, ca.data(), sizeof(double) * ca.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(b->d_step, 0, sizeof(int)) != cudaSuccess ||
      cudaMemset(b->d_cta_ns, 0, sizeof(unsigned long long) * 2 * b->cta.size()) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_CUDA, "batch_create: upload failed"));
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
    return fail(infoli__fail(INFOLI_ERR_CUDA, "batch_create: stream/event creation failed"));
  for (BatchGroup& g : b->groups)
    if (cudaStreamCreateWithPriority(&g.stream, cudaStreamNonBlocking, g.priority) != cudaSuccess ||
        cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming) != cudaSuccess)
      return fail(infoli__fail(INFOLI_ERR_CUDA, "batch_create: stream/event creation failed"));
  *out = b;
  return INFOLI_OK;
}

extern "C" int infoli_batch_set_stimulus_pulse(infoli_batch* b, int start_step, int end_step, float amp) {
  infoli__clear_error();
  if (!b) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  b->pulse_start = start_step;
  b->pulse_end = end_step;
  b->pulse_amp = amp;
  for (BatchCta& w : b->cta) {
    w.pulse_start = start_step;
    w.pulse_end = end_step;
    w.pulse_amp = amp;
  }
  BK(cudaSetDevice(b->device));
  BK(cudaStreamSynchronize(b->stream));
  BK(cudaMemcpy(b->d_cta, b->cta.data(), sizeof(BatchCta) * b->cta.size(), cudaMemcpyHostToDevice));
  return INFOLI_OK;
}

extern "C" int infoli_batch_run(infoli_batch* b, int n_steps) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_batch_run");
  if (!b || n_steps < 0) return infoli__fail(INFOLI_ERR_ARG, "batch_run: bad argument");
  BK(cudaSetDevice(b->device));
  if (b->graph_steps != n_steps) {
    // capture the group launches + the step advance once per run length
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph_exec = nullptr;
    b->graph = nullptr;
    BatchArgs a{};
    a.P = b->P;
    a.cta = b->d_cta;
    a.step = b->d_step;
    a.n_steps = n_steps;
    a.cta_ns = b->d_cta_ns;
    BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(b->fork, b->stream);
    for (const BatchGroup& g : b->groups) {
      if (e == cudaSuccess) e = cudaStreamWaitEvent(g.stream, b->fork, 0);
      if (e == cudaSuccess) e = launch_group(b, g, a);
      if (e == cudaSuccess) e = cudaEventRecord(g.done, g.stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, g.done, 0);
    }
    if (e == cudaSuccess) {
      batch_advance<<<1, 32, 0, b->stream>>>(b->d_step, n_steps);
      e = cudaGetLastError();
    }
    cudaError_t e3 = cudaStreamEndCapture(b->stream, &b->graph);
    if (e != cudaSuccess || e3 != cudaSuccess)
      return infoli__fail(INFOLI_ERR_CUDA, "batch_run: capture failed: %s / %s", cudaGetErrorString(e),
                          cudaGetErrorString(e3));
    BK(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
    b->graph_steps = n_steps;
  }
  BK(cudaEventRecord(b->ev0, b->stream));
  BK(cudaGraphLaunch(b->graph_exec, b->stream));
  BK(cudaEventRecord(b->ev1, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  BK(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  return INFOLI_OK;
}

extern "C" int infoli_batch_get_state(infoli_batch* b, float* out) {
  infoli__clear_error();
  if (!b || !out) return infoli__fail(INFOLI_ERR_ARG, "batch_get_state: bad argument");
  BK(cudaSetDevice(b->device));
  BK(cudaStreamSynchronize(b->stream));
  BK(cudaMemcpy(out, b->d_st, sizeof(float) * (size_t)INFOLI_NSTATE * b->total, cudaMemcpyDeviceToHost));
  std::vector<double> ca((size_t)b->total);
  BK(cudaMemcpy(ca.data(), b->d_ca, sizeof(double) * ca.size(), cudaMemcpyDeviceToHost));
  for (long long i = 0; i < b->total; ++i) out[4 * b->total + i] = (float)ca[(size_t)i];
  return INFOLI_OK;
}

extern "C" int infoli_batch_set_state(infoli_batch* b, const float* in) {
  infoli__clear_error();
  if (!b || !in) return infoli__fail(INFOLI_ERR_ARG, "batch_set_state: bad argument");
  BK(cudaSetDevice(b->device));
  BK(cudaStreamSynchronize(b->stream));
  BK(cudaMemcpy(b->d_st, in, sizeof(float) * (size_t)INFOLI_NSTATE * b->total, cudaMemcpyHostToDevice));
  std::vector<double> ca(in + 4 * b->total, in + 5 * b->total);
  BK(cudaMemcpy(b->d_ca, ca.data(), sizeof(double) * ca.size(), cudaMemcpyHostToDevice));
  return INFOLI_OK;
}

extern "C" int infoli_batch_info(infoli_batch* b, int* ctas, int* cluster, int* block, int64_t* cells,
                                 float* last_ms) {
  infoli__clear_error();
  if (!b) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  int cs = 1;
  for (const BatchGroup& g : b->groups) cs = std::max(cs, g.cs);
  if (ctas) *ctas = (int)b->cta.size();
  if (cluster) *cluster = cs;
  if (block) *block = b->block;
  if (cells) *cells = b->total;
  if (last_ms) *last_ms = b->last_ms;
  return INFOLI_OK;
}

extern "C" int infoli_batch_cta_info(infoli_batch* b, int* max_active_clusters, int32_t* net, int64_t* start_ns,
                                     int64_t* end_ns) {
  infoli__clear_error();
  if (!b) return infoli__fail(INFOLI_ERR_ARG, "null handle");
  if (max_active_clusters) *max_active_clusters = b->groups.empty() ? 0 : b->groups.front().max_active;
  for (size_t i = 0; i < b->cta.size(); ++i)
    if (net) net[i] = b->cta[i].net;
  if (start_ns || end_ns) {
    BK(cudaSetDevice(b->device));
    BK(cudaStreamSynchronize(b->stream));
    std::vector<unsigned long long> t(2 * b->cta.size());
    BK(cudaMemcpy(t.data(), b->d_cta_ns, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost));
    unsigned long long t0 = ~0ull;
    for (size_t i = 0; i < b->cta.size(); ++i) t0 = std::min(t0, t[2 * i]);
    for (size_t i = 0; i < b->cta.size(); ++i) {
      if (start_ns) start_ns[i] = (int64_t)(t[2 * i] - t0);
      if (end_ns) end_ns[i] = (int64_t)(t[2 * i + 1] - t0);
    }
  }
  return INFOLI_OK;
}

extern "C" int infoli_batch_destroy(infoli_batch* b) {
  infoli__clear_error();
  batch_release(b);
  return INFOLI_OK;
}

// ------------------------------------------------------------------ autotuner
// The launch layout -- cells per CTA (and with it the cluster sizes and how
// many networks share an SM) together with which networks keep their bitmask
// rows in shared memory (which in turn decides whether two 512-thread CTAs
// fit on an SM) -- is picked by timing every candidate on a trial batch.
// The trial batch is a stratified sample of the networks: sorted by size,
// m evenly spaced picks, m the smallest count whose cells reach the target
// (every SM's 1,024 threads twice over; m at most 4,096 unless the caller
// gives a cap), so the trial fills the device like the batch does and covers
// its size range.

namespace {

constexpr int kTuneMaxSample = 4096;  // sample cap when the caller gives none
constexpr int kTuneRuns = 3;           // timed runs per candidate (the best counts)
constexpr float kTuneMargin = 0.98f;   // a later candidate must be 2% faster than the pick

int tune_sample(int n_nets, const int* n_cells, int max_sample, long long target_cells, std::vector<int>& out) {
  std::vector<int> ord(n_nets);
  for (int i = 0; i < n_nets; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return n_cells[x] < n_cells[y]; });
  const int cap = std::min(max_sample > 0 ? max_sample : kTuneMaxSample, n_nets);
  // no sample of fewer than target / (largest network) networks reaches the
  // target, so the search starts there (the scan costs O(m) per count)
  long long lo = 1;
  if (target_cells > 0) lo = (target_cells + n_cells[ord.back()] - 1) / n_cells[ord.back()];
  for (int m = (int)std::min<long long>(std::max(1LL, lo), cap); m <= cap; ++m) {
    // picks (2k + 1) n_nets / (2m) are distinct because n_nets / m >= 1
    out.clear();
    long long cells = 0;
    for (int k = 0; k < m; ++k) {
      const int i = ord[(int)(((long long)(2 * k + 1) * n_nets) / (2LL * m))];
      out.push_back(i);
      cells += n_cells[i];
    }
    if (cells >= target_cells) break;
  }
  std::sort(out.begin(), out.end());  // the batch's own order
  return (int)out.size();
}

}  // namespace

extern "C" int infoli_batch_tune_sample(int n_nets, const int* n_cells, int max_sample, int64_t target_cells,
                                        int* out_idx) {
  infoli__clear_error();
  if (n_nets <= 0 || !n_cells || !out_idx) return infoli__fail(INFOLI_ERR_ARG, "batch_tune_sample: bad argument");
  std::vector<int> pick;
  const int m = tune_sample(n_nets, n_cells, max_sample, (long long)target_cells, pick);
  std::copy(pick.begin(), pick.end(), out_idx);
  return m;
}

extern "C" int infoli_batch_autotune(const infoli_batch_desc* d, int max_sample, int trial_steps,
                                     infoli_batch_tune* out) {
  infoli__clear_error();
  InfoliRange nvtx_range("infoli_batch_autotune");
  if (!d || !out || d->n_nets <= 0 || !d->n_cells || !d->params || !d->bits || !d->g ||
      (!d->init_state && !d->init_values) || trial_steps <= 0)
    return infoli__fail(INFOLI_ERR_ARG, "batch_autotune: bad argument");
  std::vector<long long> in_base(d->n_nets + 1, 0), cell_base(d->n_nets + 1, 0);
  for (int i = 0; i < d->n_nets; ++i) {
    const int n = d->n_cells[i];
    if (n <= 0 || n > 8192)
      return infoli__fail(INFOLI_ERR_ARG, "batch_autotune: network %d has %d cells (1 to 8192)", i, n);
    in_base[i + 1] = in_base[i] + (long long)n * ((n + 31) / 32);
    cell_base[i + 1] = cell_base[i] + n;
  }
  int sms = 0;
  if (cudaSetDevice(d->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device) != cudaSuccess)
    return infoli__fail(INFOLI_ERR_CUDA, "batch_autotune: no CUDA device %d", d->device);

  std::vector<int> pick;
  tune_sample(d->n_nets, d->n_cells, max_sample, 2LL * sms * 1024, pick);
  const int m = (int)pick.size();
  // the trial descriptor: the sampled networks' sizes, bitmasks, conductances
  // and initial state, laid end to end in the sample's order
  std::vector<int> sizes(m);
  std::vector<float> gs(m);
  long long words = 0, cells = 0;
  for (int k = 0; k < m; ++k) {
    sizes[k] = d->n_cells[pick[k]];
    gs[k] = d->g[pick[k]];
    words += in_base[pick[k] + 1] - in_base[pick[k]];
    cells += sizes[k];
  }
  std::vector<uint32_t> bits((size_t)words);
  std::vector<float> st(d->init_state ? (size_t)INFOLI_NSTATE * (size_t)cells : 0);
  const long long total = cell_base[d->n_nets];
  long long wo = 0, co = 0;
  for (int k = 0; k < m; ++k) {
    const int i = pick[k];
    std::copy(d->bits + in_base[i], d->bits + in_base[i + 1], bits.begin() + wo);
    wo += in_base[i + 1] - in_base[i];
    if (d->init_state)
      for (int f = 0; f < INFOLI_NSTATE; ++f)
        std::copy(d->init_state + f * total + cell_base[i], d->init_state + f * total + cell_base[i + 1],
                  st.begin() + f * cells + co);
    co += sizes[k];
  }
  infoli_batch_desc t = *d;
  t.n_nets = m;
  t.n_cells = sizes.data();
  t.bits = bits.data();
  t.g = gs.data();
  t.init_state = d->init_state ? st.data() : nullptr;

  const int cand_block[INFOLI_TUNE_CANDIDATES] = {1024, 1024, 512, 512, 512};
  const int cand_res[INFOLI_TUNE_CANDIDATES] = {INFOLI_RES_FIT, INFOLI_RES_NONE, INFOLI_RES_FIT, INFOLI_RES_OCC,
                                                INFOLI_RES_NONE};
  int best = 0;
  for (int s = 0; s < INFOLI_TUNE_CANDIDATES; ++s) {
    t.block = cand_block[s];
    t.residency = cand_res[s];
    infoli_batch* b = nullptr;
    int rc = infoli_batch_create(&t, &b);
    if (rc != INFOLI_OK) return rc;
    // the first run captures the graph for trial_steps; the best of the next
    // kTuneRuns is the candidate's time
    rc = infoli_batch_run(b, trial_steps);
    float ms = 0.0f;
    for (int k = 0; k < kTuneRuns && rc == INFOLI_OK; ++k) {
      rc = infoli_batch_run(b, trial_steps);
      if (k == 0 || b->last_ms < ms) ms = b->last_ms;
    }
    out->cand_block[s] = cand_block[s];
    out->cand_residency[s] = cand_res[s];
    out->cand_ms_per_step[s] = ms / (float)trial_steps;
    batch_release(b);  // keeps the error message of a failed run
    if (rc != INFOLI_OK) return rc;
    // a later candidate replaces the pick only when it is clearly faster:
    // trial-to-trial noise is a few percent
    if (out->cand_ms_per_step[s] < kTuneMargin * out->cand_ms_per_step[best]) best = s;
  }
  infoli__clear_error();
  out->block = cand_block[best];
  out->residency = cand_res[best];
  out->sample_nets = m;
  out->sample_cells = cells;
  return INFOLI_OK;
}

// ----------------------------------------------------------------------- lane
// The serving loop's lane: small networks, each on device buffers of its own,
// run through the batched kernel in launches of a few thousand steps; between
// launches networks join and leave.  One launch = one kernel per cluster size
// (1,024-thread CTAs, one network per cluster), the kernels running
// concurrently on one stream each, forked from and joined into the lane's
// stream.  A network's arithmetic does not depend on which others share its
// launch.

// CTAs one lane launch may hold (the server launches at most one CTA per SM)
constexpr size_t kLaneTableCtas = 1024;

struct infoli_lane {
  int device = 0;
  ModelParams P{};
  int kahan = 0;
  size_t budget = 0;  // dynamic shared memory per CTA
  cudaStream_t stream = nullptr;
  cudaStream_t gs[8] = {};
  cudaEvent_t gdone[8] = {};
  cudaEvent_t fork = nullptr, done = nullptr;
  BatchCta* h_cta = nullptr;  // pinned: the table of the launch in flight
  BatchCta* d_cta = nullptr;
  unsigned long long* d_cta_ns = nullptr;
  int* d_step = nullptr;
  size_t cap = 0;  // CTAs the table buffers hold
  bool launched = false;
};

int infoli__lane_pack_bits(int n, const int64_t* row_ptr, const int32_t* col, uint32_t* out) {
  const int wpr = (n + 31) / 32;
  std::fill(out, out + (size_t)n * (wpr + 2), 0u);
  for (int r = 0; r < n; ++r)
    for (int64_t e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
      const int s = col[e];
      if (s < 0 || s >= n) return -1;
      if (s == r) continue;  // a self edge adds f(0) * 0 = 0
      uint32_t& x = out[(size_t)(s / 32) * n + r];
      const uint32_t bit = 1u << (31 - s % 32);
      if (x & bit) return -2;  // a repeated sender cannot be one bit
      x |= bit;
    }
  return 0;
}

int infoli__lane_ctas(int n) { return (n + 1023) / 1024; }

void infoli__lane_destroy(infoli_lane* L) {
  if (!L) return;
  cudaSetDevice(L->device);
  if (L->stream) cudaStreamSynchronize(L->stream);
  if (L->h_cta) cudaFreeHost(L->h_cta);
  for (void* p : {(void*)L->d_cta, (void*)L->d_cta_ns, (void*)L->d_step})
    if (p) cudaFree(p);
  for (int k = 0; k < 8; ++k) {
    if (L->gdone[k]) cudaEventDestroy(L->gdone[k]);
    if (L->gs[k]) cudaStreamDestroy(L->gs[k]);
  }
  if (L->fork) cudaEventDestroy(L->fork);
  if (L->done) cudaEventDestroy(L->done);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
}

int infoli__lane_create(int device, const float* params, int kahan, infoli_lane** out) {
  *out = nullptr;
  infoli_lane* L = new infoli_lane();
  L->device = device;
  std::memcpy(&L->P, params, sizeof(ModelParams));
  L->kahan = kahan ? 1 : 0;
  int smem_optin = 0, prio_lo = 0, prio_hi = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess) {
    infoli__lane_destroy(L);
    return infoli__fail(INFOLI_ERR_CUDA, "lane: no CUDA device %d", device);
  }
  L->budget = (size_t)smem_optin - 1024;
  cudaError_t e = set_attrs(1024, L->budget, 8);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  for (int k = 0; k < 8 && e == cudaSuccess; ++k) {
    // larger clusters first (highest priority), as in the batch
    const int pr = std::max(prio_hi, std::min(prio_lo, prio_hi + (7 - k) * (prio_lo - prio_hi) / 8));
    e = cudaStreamCreateWithPriority(&L->gs[k], cudaStreamNonBlocking, pr);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->gdone[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc((void**)&L->d_step, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(L->d_step, 0, sizeof(int));
  // table buffers for kLaneTableCtas CTAs, allocated once: growing them later
  // would free the old ones, and cudaFree / cudaFreeHost wait for every kernel
  // on the device
  if (e == cudaSuccess) e = cudaMallocHost((void**)&L->h_cta, sizeof(BatchCta) * kLaneTableCtas);
  if (e == cudaSuccess) e = cudaMalloc((void**)&L->d_cta, sizeof(BatchCta) * kLaneTableCtas);
  if (e == cudaSuccess) e = cudaMalloc((void**)&L->d_cta_ns, sizeof(unsigned long long) * 2 * kLaneTableCtas);
  if (e == cudaSuccess) L->cap = kLaneTableCtas;
  if (e != cudaSuccess) {
    const char* msg = cudaGetErrorString(e);
    infoli__lane_destroy(L);
    return infoli__fail(INFOLI_ERR_CUDA, "lane: set-up failed: %s", msg);
  }
  *out = L;
  return INFOLI_OK;
}

void* infoli__lane_stream(infoli_lane* L) { return L ? (void*)L->stream : nullptr; }

int infoli__lane_query(infoli_lane* L) {
  if (!L || !L->launched) return 1;
  const cudaError_t e = cudaEventQuery(L->done);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return infoli__fail(INFOLI_ERR_CUDA, "lane: %s", cudaGetErrorString(e));
}

int infoli__lane_launch(infoli_lane* L, const LaneNet* nets, int count) {
  if (!L || (count > 0 && !nets)) return infoli__fail(INFOLI_ERR_ARG, "lane_launch: bad argument");
  BK(cudaSetDevice(L->device));
  if (L->launched) BK(cudaEventSynchronize(L->done));  // the table buffers are reused
  L->launched = false;
  size_t total = 0;
  for (int i = 0; i < count; ++i) {
    if (nets[i].n <= 0 || nets[i].n > kLaneMaxCells || nets[i].n_steps < 0 || nets[i].step0 < 0)
      return infoli__fail(INFOLI_ERR_ARG, "lane_launch: network %d (%d cells, %d steps)", i, nets[i].n,
                          nets[i].n_steps);
    total += (size_t)infoli__lane_ctas(nets[i].n);
  }
  if (total == 0) return INFOLI_OK;
  if (total > L->cap)
    return infoli__fail(INFOLI_ERR_CAPACITY, "lane_launch: %zu CTAs (at most %zu per launch)", total, L->cap);
  struct Grp {
    int off = 0, grid = 0, vcap = 0, res_words = 0;
    size_t smem = 0;
  } grp[8];
  size_t off = 0;
  for (int cs = 8; cs >= 1; --cs) {
    Grp& g = grp[cs - 1];
    g.off = (int)off;
    int nmax = 0;
    for (int i = 0; i < count; ++i)
      if (infoli__lane_ctas(nets[i].n) == cs) nmax = std::max(nmax, nets[i].n);
    if (nmax == 0) continue;
    g.vcap = ((nmax + 31) / 32) * 32 + 32;
    const size_t vbytes = 2 * sizeof(float) * (size_t)g.vcap;
    int res_rows = 0;
    for (int i = 0; i < count; ++i) {
      const int n = nets[i].n;
      if (infoli__lane_ctas(n) != cs) continue;
      const int wr = (n + 31) / 32 + 2;
      if (vbytes + sizeof(uint32_t) * (size_t)wr * 1024 <= L->budget) res_rows = std::max(res_rows, wr);
    }
    g.res_words = res_rows * 1024;
    g.smem = vbytes + sizeof(uint32_t) * (size_t)g.res_words;
    for (int i = 0; i < count; ++i) {
      const LaneNet& q = nets[i];
      if (infoli__lane_ctas(q.n) != cs) continue;
      const int per = (q.n + cs - 1) / cs;
      for (int k = 0; k < cs; ++k) {
        BatchCta& w = L->h_cta[off++];
        w = BatchCta{};
        w.net = i;
        w.rank = k;
        w.ncta = cs;
        w.rank0 = 0;
        w.cbeg = std::min(q.n, k * per);
        w.ncell = std::min(q.n, (k + 1) * per) - w.cbeg;
        w.n = q.n;
        w.wpr = (q.n + 31) / 32;
        w.st = q.st;
        w.ca = q.ca;
        w.bits = q.bits;
        w.T = q.n;
        w.cell_base = 0;
        w.g = q.g;
        w.resident = (w.wpr + 2) * 1024 <= g.res_words ? 1 : 0;
        w.cl_sync = cs > 1 ? 1 : 0;
        w.n_steps = q.n_steps;
        w.step0 = q.step0;
        w.pulse_start = q.pulse_start;
        w.pulse_end = q.pulse_end;
        w.pulse_amp = q.pulse_amp;
      }
    }
    g.grid = (int)off - g.off;
  }
  BK(cudaMemcpyAsync(L->d_cta, L->h_cta, sizeof(BatchCta) * total, cudaMemcpyHostToDevice, L->stream));
  BK(cudaEventRecord(L->fork, L->stream));
  for (int cs = 8; cs >= 1; --cs) {
    const Grp& g = grp[cs - 1];
    if (g.grid == 0) continue;
    BatchArgs a{};
    a.P = L->P;
    a.cta = L->d_cta + g.off;
    a.vcap = g.vcap;
    a.res_words = g.res_words;
    a.step = L->d_step;
    a.n_steps = 0;
    a.cta_ns = L->d_cta_ns + 2 * (size_t)g.off;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at[2];
    fill_config(cfg, at, g.grid, 1024, cs, g.smem, 0, L->gs[cs - 1]);
    cfg.numAttrs = 1;  // stream priority comes from the stream
    BK(cudaStreamWaitEvent(L->gs[cs - 1], L->fork, 0));
    BK(L->kahan ? cudaLaunchKernelEx(&cfg, batch_kernel<1024, true>, a)
                : cudaLaunchKernelEx(&cfg, batch_kernel<1024, false>, a));
    BK(cudaEventRecord(L->gdone[cs - 1], L->gs[cs - 1]));
    BK(cudaStreamWaitEvent(L->stream, L->gdone[cs - 1], 0));
  }
  BK(cudaEventRecord(L->done, L->stream));
  L->launched = true;
  return INFOLI_OK;
}
