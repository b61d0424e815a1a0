// Persistent, cooperative step kernel: gap-junction coupling fused with the
// 3-compartment cell update, one grid barrier per simulated step.
//
// Per step, each CTA:
//   1. stages the V_dend tiles its receivers read (bulk async copy global ->
//      shared, mbarrier completion, double-buffered when there are several);
//   2. phase A -- coupling (src/openmp/infoli.c:496-520): each warp reduces
//      one chunk of <= 128 edges of one receiver:
//          I_c += g * (0.8 exp(-V^2/100) + 0.2) * V,   V = V_dend[c] - V_dend[n]
//      exp on the SFU (ex2.approx of the base-2 argument), lanes accumulate in
//      FP32 (optionally Kahan-compensated), warp shuffles reduce, lane 0 writes
//      the chunk's partial sum to shared memory;
//   3. phase B -- one thread per owned cell adds its receiver's partials in
//      sender order and runs the fused compartment update
//      (src/openmp/infoli.c:556-675) on register-resident state, then writes
//      the new V_dend into the other half of the double buffer;
//   4. grid barrier (release/acquire counter, bounded wait: on timeout the
//      kernel records an error and every CTA returns).
#include <cstdio>

#include "infoli_kernels.cuh"
#include "infoli_ptx.cuh"

namespace infoli {

namespace {

constexpr float kNegLog2eOver100 = -0.014426950408889634f;  // -log2(e)/100

// Wait for phase `parity` of an mbarrier, bounded by the launch's timeout.
__device__ __forceinline__ bool wait_tile(const StepArgs& a, uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer_ns() - t0 > a.timeout_ns) {
      atomicCAS(a.err, 0, DEV_ERR_COPY_TIMEOUT);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void issue_tile(const StepArgs& a, const float* vcur, const TileDesc& td, float* dst,
                                           uint64_t* bar) {
  const unsigned bytes = (unsigned)td.nfloats * 4u;
  mbar_arrive_expect_tx(bar, bytes);
  bulk_g2s(dst, vcur + td.lo, bytes, bar);
}

// Grid barrier: arrive on a monotonically increasing counter, wait until it
// reaches `target`.  Returns false (and makes the whole CTA return) when the
// wait gives up or another CTA has recorded an error.
__device__ __forceinline__ bool grid_sync(const StepArgs& a, unsigned target, volatile int* s_abort,
                                          uint64_t* t_arrive) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (t_arrive) *t_arrive = globaltimer_ns();
    __threadfence();
    red_release_gpu_add(a.bar, 1u);
    if (ld_acquire_gpu(a.bar) < target) {
      const uint64_t t0 = globaltimer_ns();
      while (ld_acquire_gpu(a.bar) < target) {
        if (ld_relaxed_gpu(a.err) != 0) {
          *s_abort = 1;
          break;
        }
        if (globaltimer_ns() - t0 > a.timeout_ns) {
          atomicCAS(a.err, 0, DEV_ERR_BARRIER_TIMEOUT);
          *s_abort = 1;
          break;
        }
      }
    }
  }
  __syncthreads();
  return *s_abort == 0;
}

template <bool KAHAN, bool EDGE_G>
__global__ void __launch_bounds__(1024, 1) step_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  const SmemShape shp = a.shape;
  const SmemLayout L = smem_layout(shp);
  float* tbuf = reinterpret_cast<float*>(smem_raw + L.tiles);
  float* vown = reinterpret_cast<float*>(smem_raw + L.vown);
  float* part = reinterpret_cast<float*>(smem_raw + L.part);
  float* partc = reinterpret_cast<float*>(smem_raw + L.partc);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + L.mbar);

  const CtaWork w = a.cta[blockIdx.x];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const bool owner = tid < w.n_cells;
  const int cell = w.cell_begin + tid;
  const long long np = a.n_pad;
  const int tile_cap = shp.tile_cap;
  const int nbuf = shp.nbuf;

  // ---- static work: either resident in shared memory or read from global.
  // Indices below are relative to the CTA's first chunk / edge.
  const TileDesc* tiles = a.tiles + w.tile_begin;
  const ChunkDesc* chunks = a.chunks;
  const uint16_t* edges = a.edges;
  const float* edge_g = a.edge_g;
  int chunk0 = 0, edge0 = 0;
  if (w.n_tiles > 0) {
    chunk0 = tiles[0].chunk_begin;
    const int chunk1 = tiles[w.n_tiles - 1].chunk_end;
    edge0 = chunk1 > chunk0 ? a.chunks[chunk0].edge_begin : 0;
    const bool resident = shp.res_chunks > 0;
    if (resident) {
      TileDesc* s_t = reinterpret_cast<TileDesc*>(smem_raw + L.tdesc);
      ChunkDesc* s_c = reinterpret_cast<ChunkDesc*>(smem_raw + L.chunks);
      uint16_t* s_e = reinterpret_cast<uint16_t*>(smem_raw + L.edges);
      float* s_g = reinterpret_cast<float*>(smem_raw + L.eg);
      const int nch = chunk1 - chunk0;
      const int ned = nch > 0 ? a.chunks[chunk1 - 1].edge_begin + a.chunks[chunk1 - 1].count - edge0 : 0;
      for (int i = tid; i < w.n_tiles; i += blockDim.x) {
        TileDesc td = tiles[i];
        td.chunk_begin -= chunk0;
        td.chunk_end -= chunk0;
        s_t[i] = td;
      }
      for (int i = tid; i < nch; i += blockDim.x) {
        ChunkDesc c = a.chunks[chunk0 + i];
        c.edge_begin -= edge0;
        s_c[i] = c;
      }
      for (int i = tid; i < ned; i += blockDim.x) {
        s_e[i] = a.edges[edge0 + i];
        if (EDGE_G) s_g[i] = a.edge_g[edge0 + i];
      }
      tiles = s_t;
      chunks = s_c;
      edges = s_e;
      edge_g = s_g;
      chunk0 = 0;
      edge0 = 0;
    } else {
      chunks = a.chunks + chunk0;
      edges = a.edges + edge0;
      if (EDGE_G) edge_g = a.edge_g + edge0;
    }
  }

  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }

  CellState cs;
  int2 slots = make_int2(0, 0);
  float gscale = a.g_uniform;
  float my_amp = 0.0f;
  int my_onset = 0, my_off = 0;
  if (owner) {
    const float* st = a.st;
    cs.Vd = a.vd[a.step0 & 1][cell];
    cs.Vs = st[F_VS * np + cell];
    cs.Va = st[F_VA * np + cell];
    cs.q = st[F_Q * np + cell];
    cs.r = st[F_R * np + cell];
    cs.s = st[F_S * np + cell];
    cs.Ca = a.ca[cell];
    cs.ICaH = st[F_ICAH * np + cell];
    cs.gCaL = st[F_GCAL * np + cell];
    cs.k = st[F_K * np + cell];
    cs.l = st[F_L * np + cell];
    cs.m = st[F_M * np + cell];
    cs.h = st[F_H * np + cell];
    cs.n = st[F_N * np + cell];
    cs.p = st[F_P * np + cell];
    cs.xs = st[F_XS * np + cell];
    cs.ma = st[F_MA * np + cell];
    cs.ha = st[F_HA * np + cell];
    cs.xa = st[F_XA * np + cell];
    slots = a.cell_slots[cell];
    if (a.cell_g) gscale = a.cell_g[cell];
    if (a.stim_kind == STIM_CELL) {
      my_amp = a.cell_amp[cell];
      my_onset = a.cell_onset[cell];
    }
    if (a.cell_step_off) my_off = a.cell_step_off[cell];
    vown[tid] = cs.Vd;
  }
  __syncthreads();

  const bool prof = a.prof != nullptr && tid == 0;
  __shared__ unsigned long long s_prof[5];
  if (prof) s_prof[0] = s_prof[1] = s_prof[2] = s_prof[3] = s_prof[4] = 0;
  uint64_t t_step = prof ? globaltimer_ns() : 0;

  unsigned nload = 0;  // bulk tile loads issued so far (same value in every thread)
  int row = 0;
  unsigned bar_target = 0;
  for (int t = 0; t < a.n_steps; ++t) {
    const int step = a.step0 + t;
    const float* vcur = a.vd[step & 1];
    uint64_t t_ready = 0;

    // ---------------- stage tiles + phase A (coupling)
    if (w.n_tiles > 0) {
      if (tid == 0) {
        fence_proxy_async_global();
        fence_proxy_async_smem();
        issue_tile(a, vcur, tiles[0], tbuf + (nload % nbuf) * tile_cap, &mbar[nload % nbuf]);
      }
      for (int j = 0; j < w.n_tiles; ++j) {
        const TileDesc td = tiles[j];
        const unsigned k = nload + j;
        const int b = (int)(k % (unsigned)nbuf);
        float* buf = tbuf + b * tile_cap;
        if (tid == 0 && j > 0 && nbuf == 1) {
          fence_proxy_async_smem();
          issue_tile(a, vcur, td, buf, &mbar[b]);
        }
        if (tid == 0 && j + 1 < w.n_tiles && nbuf == 2) {
          fence_proxy_async_smem();
          const int b1 = (int)((k + 1) & 1u);
          issue_tile(a, vcur, tiles[j + 1], tbuf + b1 * tile_cap, &mbar[b1]);
        }
        if (!wait_tile(a, &mbar[b], (k / (unsigned)nbuf) & 1u)) s_abort = 1;
        if (prof && j == 0) t_ready = globaltimer_ns();

        for (int ci = td.chunk_begin - chunk0 + warp; ci < td.chunk_end - chunk0; ci += nwarps) {
          const ChunkDesc c = chunks[ci];
          const float vc = vown[c.recv];
          const int eb = c.edge_begin - edge0;
          float acc = 0.0f, comp = 0.0f;
#pragma unroll 4
          for (int u = lane; u < c.count; u += 32) {
            const int e = eb + u;
            const float V = vc - buf[edges[e]];
            const float f = fmaf(0.8f, ex2_approx((V * V) * kNegLog2eOver100), 0.2f);
            float term;
            if (EDGE_G)
              term = (edge_g[e] * f) * V;
            else
              term = f * V;
            if (KAHAN) {
              const float y = term - comp;
              const float s = acc + y;
              comp = (s - acc) - y;
              acc = s;
            } else {
              acc += term;
            }
          }
          if (KAHAN) {
            // carry the compensation separately through the tree
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
              acc += __shfl_xor_sync(0xffffffffu, acc, o);
              comp += __shfl_xor_sync(0xffffffffu, comp, o);
            }
            if (lane == 0) {
              part[c.slot] = acc;
              partc[c.slot] = comp;
            }
          } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) part[c.slot] = acc;
          }
        }
        __syncthreads();
      }
      nload += w.n_tiles;
    } else if (prof) {
      t_ready = globaltimer_ns();
    }
    uint64_t t_coupled = prof ? globaltimer_ns() : 0;

    // ---------------- phase B (fused compartment update)
    if (owner) {
      float ic;
      if (KAHAN) {
        float s = 0.0f, cmp = 0.0f;
        for (int q = 0; q < slots.y; ++q) {
          const float y = part[slots.x + q] - (partc[slots.x + q] + cmp);
          const float tt = s + y;
          cmp = (tt - s) - y;
          s = tt;
        }
        ic = s;
      } else {
        ic = 0.0f;
        for (int q = 0; q < slots.y; ++q) ic += part[slots.x + q];
      }
      if (!EDGE_G) ic *= gscale;
      const int ls = step + my_off;
      float iapp;
      if (a.stim_kind == STIM_PULSE)
        iapp = (ls >= a.stim_start && ls < a.stim_end) ? a.stim_amp : 0.0f;
      else if (a.stim_kind == STIM_CELL)
        iapp = (ls >= my_onset && ls < my_onset + a.stim_dur) ? my_amp : 0.0f;
      else
        iapp = a.stim_table[(size_t)t * np + cell];
      cell_step(a.P, cs, ic, iapp);
      a.vd[(step + 1) & 1][cell] = cs.Vd;
      vown[tid] = cs.Vd;
      if (a.trace_every > 0 && (step % a.trace_every) == 0) {
        float* tr = a.trace + (size_t)row * a.trace_nq * np + cell;
        int qi = 0;
        if (a.trace_mask & TRACE_AXON) tr[(qi++) * np] = cs.Va;
        if (a.trace_mask & TRACE_SOMA) tr[(qi++) * np] = cs.Vs;
        if (a.trace_mask & TRACE_DEND) tr[(qi++) * np] = cs.Vd;
      }
    }
    if (a.trace_every > 0 && (step % a.trace_every) == 0) ++row;

    if (t + 1 < a.n_steps) {
      bar_target += gridDim.x;
      uint64_t t_arrive = 0;
      const bool ok = grid_sync(a, bar_target, &s_abort, prof ? &t_arrive : nullptr);
      if (prof) {
        const uint64_t t_done = globaltimer_ns();
        s_prof[0] += t_ready - t_step;
        s_prof[1] += t_coupled - t_ready;
        s_prof[2] += t_arrive - t_coupled;
        s_prof[3] += t_done - t_arrive;
        s_prof[4] += 1;
        t_step = t_done;
      }
      if (!ok) break;
    }
  }
  if (prof) {
    unsigned long long* pr = a.prof + (size_t)blockIdx.x * kProfSlots;
    atomicAdd(pr + PROF_STAGE, s_prof[0]);
    atomicAdd(pr + PROF_COUPLE, s_prof[1]);
    atomicAdd(pr + PROF_UPDATE, s_prof[2]);
    atomicAdd(pr + PROF_BARRIER, s_prof[3]);
    atomicAdd(pr + PROF_STEPS, s_prof[4]);
  }

  if (owner) {
    float* st = a.st;
    st[F_VS * np + cell] = cs.Vs;
    st[F_VA * np + cell] = cs.Va;
    st[F_Q * np + cell] = cs.q;
    st[F_R * np + cell] = cs.r;
    st[F_S * np + cell] = cs.s;
    a.ca[cell] = cs.Ca;
    st[F_ICAH * np + cell] = cs.ICaH;
    st[F_K * np + cell] = cs.k;
    st[F_L * np + cell] = cs.l;
    st[F_M * np + cell] = cs.m;
    st[F_H * np + cell] = cs.h;
    st[F_N * np + cell] = cs.n;
    st[F_P * np + cell] = cs.p;
    st[F_XS * np + cell] = cs.xs;
    st[F_MA * np + cell] = cs.ma;
    st[F_HA * np + cell] = cs.ha;
    st[F_XA * np + cell] = cs.xa;
  }
}

template <bool K, bool G>
cudaError_t launch_variant(const StepArgs& a, int grid, int threads, size_t smem, cudaStream_t stream) {
  auto fn = step_kernel<K, G>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(threads), args, smem, stream);
}

}  // namespace

size_t step_kernel_smem(const StepArgs& a) { return smem_layout(a.shape).total; }

cudaError_t launch_step_kernel(const StepArgs& a, int grid, int threads, cudaStream_t stream) {
  const size_t smem = step_kernel_smem(a);
  const bool g = a.edge_g != nullptr;
  if (threads != a.shape.threads) return cudaErrorInvalidValue;
  if (a.shape.kahan) return g ? launch_variant<true, true>(a, grid, threads, smem, stream)
                        : launch_variant<true, false>(a, grid, threads, smem, stream);
  return g ? launch_variant<false, true>(a, grid, threads, smem, stream)
           : launch_variant<false, false>(a, grid, threads, smem, stream);
}

int max_coresident_ctas(int threads, size_t smem) {
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  auto fn = step_kernel<false, false>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess) return 0;
  return per_sm * nsm;
}

}  // namespace infoli
