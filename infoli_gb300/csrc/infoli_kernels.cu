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
// Stamped plans keep V_dend x kVScale in the window copy and the scaled-V cell
// array (kVScale^2 = log2(e) / 100): a coupling term's exponent is then
// -(dV')^2 with dV' = kVScale dV, one multiply less per edge; the partial sums
// are scaled back once per receiver.
constexpr float kVScale = 0.12011224087864497f;
constexpr float kInvVScale = 8.325546111576978f;

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
    if (t_arrive) *t_arrive = clock64();
    __threadfence();
    if ((int)blockIdx.x != a.stall_cta) red_release_gpu_add(a.bar, 1u);
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


// Gate state of local cell r from / to shared memory (field f at
// sG[f * cap + r]), only the fields the units in `mask` use.
__device__ __forceinline__ Gates load_gates(const float* sG, const double* sCa, int cap, int r, unsigned mask) {
  Gates g;
  if (mask & 0x01u) g.q = sG[F_Q * cap + r];
  if (mask & 0x02u) {
    g.r = sG[F_R * cap + r];
    g.s = sG[F_S * cap + r];
    g.Ca = sCa[r];
    g.ICaH = sG[F_ICAH * cap + r];
  }
  if (mask & 0x04u) {
    g.k = sG[F_K * cap + r];
    g.l = sG[F_L * cap + r];
    g.gCaL = sG[F_GCAL * cap + r];
  }
  if (mask & 0x08u) g.h = sG[F_H * cap + r];
  if (mask & 0x10u) {
    g.n = sG[F_N * cap + r];
    g.p = sG[F_P * cap + r];
  }
  if (mask & 0x20u) g.xs = sG[F_XS * cap + r];
  if (mask & 0x40u) g.ha = sG[F_HA * cap + r];
  if (mask & 0x80u) g.xa = sG[F_XA * cap + r];
  return g;
}

__device__ __forceinline__ void store_gates(float* sG, double* sCa, int cap, int r, unsigned mask, const Gates& g) {
  if (mask & 0x01u) sG[F_Q * cap + r] = g.q;
  if (mask & 0x02u) {
    sG[F_R * cap + r] = g.r;
    sG[F_S * cap + r] = g.s;
    sCa[r] = g.Ca;
    sG[F_ICAH * cap + r] = g.ICaH;
  }
  if (mask & 0x04u) {
    sG[F_K * cap + r] = g.k;
    sG[F_L * cap + r] = g.l;
  }
  if (mask & 0x08u) {
    sG[F_M * cap + r] = g.m;
    sG[F_H * cap + r] = g.h;
  }
  if (mask & 0x10u) {
    sG[F_N * cap + r] = g.n;
    sG[F_P * cap + r] = g.p;
  }
  if (mask & 0x20u) sG[F_XS * cap + r] = g.xs;
  if (mask & 0x40u) {
    sG[F_MA * cap + r] = g.ma;
    sG[F_HA * cap + r] = g.ha;
  }
  if (mask & 0x80u) sG[F_XA * cap + r] = g.xa;
}

// Trace rows fall on the steps that are multiples of trace_every.  A
// countdown per thread replaces a per-step integer division (it sat on the
// voltage threads' path every step).
struct TraceClock {
  int every, left;
  __device__ TraceClock(int every_, int step0)
      : every(every_), left(every_ > 0 ? (every_ - step0 % every_) % every_ : -1) {}
  // true on a trace step; advances to the next step
  __device__ bool take() {
    const bool now = left == 0;
    if (every > 0) left = now ? every - 1 : left - 1;
    return now;
  }
};

__device__ __forceinline__ unsigned long long pack_stamp(float v, unsigned stamp) {
  return ((unsigned long long)stamp << 32) | (unsigned long long)__float_as_uint(v);
}

// Stamped exchange.  A CTA's window is one flat index space: word i <
// tile_words is the V_dend of its i-th unique sender (ascending cell ids,
// held in shared memory; the value lands at float i of the window buffer),
// word i >= tile_words is progress probe i - tile_words (checked, not
// stored).  Words of cells >= n_cells are never published and read as 0.
// Polling thread pt of T takes words pt, pt + T, ... in batches of NB loads
// in flight (the step kernel's template parameter: kPollBatchSmall when every
// polling thread has at most that many words, else kPollBatch).  A batch can
// be issued early and finished later (the loads overlap other work); every
// wait is bounded by the launch's timeout (error recorded, false returned).
// The small batch is the plan's common case and its code is much shorter:
// on the 10k grid (at most 1,272 words per CTA, 512 threads) 3 slots against
// 8 took the step from 4.35 to 4.03 us with Kahan sums and from 3.93 to 3.78
// without; the issue of the loads, not their round trip, was the larger part
// of the poll.
constexpr int kPollBatch = 8;
constexpr int kPollBatchSmall = 3;

struct PollWindow {
  const int* cells;  // the window's sender ids (shared memory)
  const int* probes;
  int n_probes;
  int tile_words;
  int total;
};

template <int NB>
struct PollBatchT {
  unsigned long long w[NB];
  int cell[NB];
  int dst[NB];  // shared-memory word, or -1 for a probe
  unsigned pend;
};

// Uncompensated stamped kernels issue the first poll batch of every thread
// before the gate units and finish it after them (kPollEarly loads per
// thread, 0 = off), so the loads' round trip overlaps the units.  Only the
// loaded words and the pending mask stay live across the units; each word's
// cell and window slot are read again from the window (shared memory) when
// they are needed.  Measured on the 10k grid: 3.93 against 4.10 us per step
// (the exchange wait falls by a third, the units slow down under the loads
// in flight); with Kahan sums the step does not gain (4.52 against 4.50 us
// with per-term compensation, 4.347 against 4.352 with two-term blocks, 4.08
// against 4.08 median with the 3-slot poll batch), so Kahan kernels poll after
// the units.  Two loads
// per thread leave part of the window to a second round trip (4.56 us); four
// spill.
#ifndef INFOLI_POLL_EARLY
#define INFOLI_POLL_EARLY 3
#endif
// Kahan stamped coupling: compensation over two-term blocks (1, the
// default) or over every term (0).  Measured on the 10k grid: 4.35 against
// 4.50 us per step, the same error against the FP64 oracle (4.33e-5 mV).
#ifndef INFOLI_KAHAN_BLOCK
#define INFOLI_KAHAN_BLOCK 1
#endif
constexpr int kPollEarly = INFOLI_POLL_EARLY;

template <int NB>
struct PollLean {
  unsigned long long w[NB];
  unsigned pend;
};

__device__ __forceinline__ int window_cell(const PollWindow& pw, int i, int* dst) {
  if (i >= pw.tile_words) {
    *dst = -1;
    return pw.probes[i - pw.tile_words];
  }
  *dst = i;
  return pw.cells[i];
}

// tbuf receives each word's V_dend x kVScale at its window index and, when
// dup > 0, again at dup + index (the bank-shifted second copy).
template <int NB>
__device__ __forceinline__ void poll_issue(const StepArgs& a, const unsigned long long* src, const PollWindow& pw,
                                           int base, int T, float* tbuf, int dup, PollBatchT<NB>& b) {
  b.pend = 0;
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    const int i = base + k * T;
    b.cell[k] = 0;
    b.dst[k] = -1;
    b.w[k] = 0;
    if (i < pw.total) {
      const int c = window_cell(pw, i, &b.dst[k]);
      if (c < a.n_cells) {
        b.cell[k] = c;
        b.pend |= 1u << k;
      } else if (b.dst[k] >= 0) {
        tbuf[b.dst[k]] = 0.0f;
        if (dup) tbuf[dup + b.dst[k]] = 0.0f;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NB; ++k)
    if ((b.pend >> k) & 1u) b.w[k] = ld_poll_u64(src + b.cell[k]);
}

// Lean batch: words base, base + T, ... (see PollLean).
template <int NB>
__device__ __forceinline__ void poll_issue_lean(const StepArgs& a, const unsigned long long* src,
                                                const PollWindow& pw, int base, int T, float* tbuf, int dup,
                                                PollLean<NB>& b) {
  b.pend = 0;
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    const int i = base + k * T;
    b.w[k] = 0;
    if (i < pw.total) {
      int dst;
      const int c = window_cell(pw, i, &dst);
      if (c < a.n_cells) {
        b.pend |= 1u << k;
        b.w[k] = ld_poll_u64(src + c);
      } else if (dst >= 0) {
        tbuf[dst] = 0.0f;
        if (dup) tbuf[dup + dst] = 0.0f;
      }
    }
  }
}

template <int NB>
__device__ __forceinline__ bool poll_finish_lean(const StepArgs& a, const unsigned long long* src,
                                                 const PollWindow& pw, int base, int T, float* tbuf, int dup,
                                                 unsigned want, PollLean<NB>& b, uint64_t& t0) {
  while (true) {
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      if (((b.pend >> k) & 1u) && (unsigned)(b.w[k] >> 32) == want) {
        const int i = base + k * T;
        if (i < pw.tile_words) {
          const float v = __uint_as_float((unsigned)b.w[k]) * kVScale;
          tbuf[i] = v;
          if (dup) tbuf[dup + i] = v;
        }
        b.pend &= ~(1u << k);
      }
    }
    if (!b.pend) return true;
    const uint64_t now = globaltimer_ns();
    if (t0 == 0) {
      t0 = now;
    } else if (now - t0 > a.timeout_ns || ld_relaxed_gpu(a.err) != 0) {
      atomicCAS(a.err, 0, DEV_ERR_STAMP_TIMEOUT);
      return false;
    }
#pragma unroll
    for (int k = 0; k < NB; ++k)
      if ((b.pend >> k) & 1u) {
        int dst;
        b.w[k] = ld_poll_u64(src + window_cell(pw, base + k * T, &dst));
      }
  }
}

// Takes the words of batch b whose stamp is `want` (their values into tbuf)
// and clears their pending bits; true when none is left.
template <int NB>
__device__ __forceinline__ bool poll_take(float* tbuf, int dup, unsigned want, PollBatchT<NB>& b) {
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    if (((b.pend >> k) & 1u) && (unsigned)(b.w[k] >> 32) == want) {
      if (b.dst[k] >= 0) {
        const float v = __uint_as_float((unsigned)b.w[k]) * kVScale;
        tbuf[b.dst[k]] = v;
        if (dup) tbuf[dup + b.dst[k]] = v;
      }
      b.pend &= ~(1u << k);
    }
  }
  return b.pend == 0;
}

// Reloads the pending words of b until all carry `want` (bounded by the
// launch's timeout: error recorded, false returned).
template <int NB>
__device__ __forceinline__ bool poll_retry(const StepArgs& a, const unsigned long long* src, float* tbuf, int dup,
                                           unsigned want, PollBatchT<NB>& b, uint64_t& t0) {
  while (true) {
    const uint64_t now = globaltimer_ns();
    if (t0 == 0) {
      t0 = now;
    } else if (now - t0 > a.timeout_ns || ld_relaxed_gpu(a.err) != 0) {
      atomicCAS(a.err, 0, DEV_ERR_STAMP_TIMEOUT);
      return false;
    }
#pragma unroll
    for (int k = 0; k < NB; ++k)
      if ((b.pend >> k) & 1u) b.w[k] = ld_poll_u64(src + b.cell[k]);
    if (poll_take<NB>(tbuf, dup, want, b)) return true;
  }
}

// The same as a call: the retry loop's code leaves the step loop's hot path.
template <int NB>
__device__ __noinline__ bool poll_retry_call(const StepArgs* a, const unsigned long long* src, float* tbuf, int dup,
                                             unsigned want, PollBatchT<NB> b, uint64_t* t0) {
  return poll_retry<NB>(*a, src, tbuf, dup, want, b, *t0);
}

// First look at an issued batch, then the retry loop for words that are not
// yet current.  OUTLINE runs the retry loop as a call: measured on the 10k
// grid, the Kahan kernel gains (4.08 -> 3.98 us per step, median) while the
// uncompensated one loses (3.81 -> 3.95 us) from the call's effect on its
// register allocation, so only the Kahan kernels use it (with the small
// batch: the 8-slot batch passed to the call spills).
template <int NB, bool OUTLINE>
__device__ __forceinline__ bool poll_finish(const StepArgs& a, const unsigned long long* src, float* tbuf, int dup,
                                            unsigned want, PollBatchT<NB>& b, uint64_t& t0) {
  if (poll_take<NB>(tbuf, dup, want, b)) return true;
  if (OUTLINE) return poll_retry_call<NB>(&a, src, tbuf, dup, want, b, &t0);
  return poll_retry<NB>(a, src, tbuf, dup, want, b, t0);
}

// Phase A of stamped plans (packed lane-chunk layout, all in shared memory):
// warp w takes groups w, w + nwarps, ... < ngroups; lane l of the warp owns
// lane-chunk l of the group (up to kLaneEdges edges of one receiver) and
// reduces it alone -- no cross-lane reduction.  Each 8-byte load brings the
// lane's next four byte offsets; padding entries address the receiver's own
// V_dend and add exactly 0.  Two accumulators (even / odd entries) shorten
// the dependent add chain; they are combined in a fixed order.
template <bool KAHAN, bool EDGE_G>
__device__ __forceinline__ void couple_packed(const unsigned char* sm, const SmemLayout& L, int ngroups,
                                              const float* sVd, float* part, float* partc, int warp, int nwarps,
                                              int lane) {
  const int2* gd = reinterpret_cast<const int2*>(sm + L.chunks);
  const uint2* ent = reinterpret_cast<const uint2*>(sm + L.edges);
  const float4* gv = reinterpret_cast<const float4*>(sm + L.eg);
  if (!KAHAN) {
    // Paired FP32 (f32x2) form: the two accumulators take edges j = 0, 2 and
    // j = 1, 3 of every quad, so one paired instruction does both.  It runs
    // on negated values (x - vc = -V exactly; fma(f, -V, -acc) = -fma(f, V,
    // acc) under round-to-nearest), which needs no paired subtraction, and
    // flips the sign once per receiver: the same operations in the same
    // order as the scalar form.
    const float2 c08 = make_float2(0.8f, 0.8f), c02 = make_float2(0.2f, 0.2f);
    for (int gi = warp; gi < ngroups; gi += nwarps) {
      const int2 d = gd[gi * 32 + lane];  // {slot, recv}
      const float nvc = -sVd[d.y];
      const float2 nvc2 = make_float2(nvc, nvc);
      float2 nacc = make_float2(-0.0f, -0.0f);
#pragma unroll
      for (int kq = 0; kq < kQuads; ++kq) {
        const int qi = (gi * kQuads + kq) * 32 + lane;
        const uint2 o = ent[qi];
        float4 g4 = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        if (EDGE_G) g4 = gv[qi];
        const unsigned off[4] = {o.x & 0xffffu, o.x >> 16, o.y & 0xffffu, o.y >> 16};
        const float2 gg[2] = {make_float2(g4.x, g4.y), make_float2(g4.z, g4.w)};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float2 x = make_float2(*reinterpret_cast<const float*>(sm + off[2 * h]),
                                       *reinterpret_cast<const float*>(sm + off[2 * h + 1]));
          const float2 nv = __fadd2_rn(x, nvc2);  // -V, scaled by kVScale
          const float2 sq = __fmul2_rn(nv, nv);
          const float2 e = make_float2(ex2_approx(-sq.x), ex2_approx(-sq.y));
          float2 f = __ffma2_rn(c08, e, c02);
          if (EDGE_G) f = __fmul2_rn(gg[h], f);
          nacc = __ffma2_rn(f, nv, nacc);
        }
      }
      part[d.x] = -(nacc.x + nacc.y);
    }
    return;
  }
  {
    // Kahan-compensated paired form (over two-term blocks by default: each
    // accumulator's terms of a quad are added first, the block sum is then
    // Kahan-added, see INFOLI_KAHAN_BLOCK).  Same sign trick: the
    // accumulators hold -sum while the compensations c hold +c, so each Kahan
    // step
    //   y = term - c,  s = acc + y,  c = (s - acc) - y,  acc = s
    // becomes, on negated terms nt = -term and nacc = -acc,
    //   ny = fma(f, -V, c),  ns = nacc + ny,  c = ny - (ns - nacc)
    // (each an exact negation of the scalar step under round-to-nearest; the
    // subtractions are fma with -1, which rounds once like a subtraction).
    // The two accumulators are merged with an error-free TwoSum whose error
    // joins the compensation, so the lane's partial and its compensation
    // carry the whole chunk.
    const float2 c08 = make_float2(0.8f, 0.8f), c02 = make_float2(0.2f, 0.2f);
    const float2 m1 = make_float2(-1.0f, -1.0f);
    for (int gi = warp; gi < ngroups; gi += nwarps) {
      const int2 d = gd[gi * 32 + lane];  // {slot, recv}
      const float nvc = -sVd[d.y];
      const float2 nvc2 = make_float2(nvc, nvc);
      float2 nacc = make_float2(-0.0f, -0.0f);
      float2 cmp = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int kq = 0; kq < kQuads; ++kq) {
        const int qi = (gi * kQuads + kq) * 32 + lane;
        const uint2 o = ent[qi];
        float4 g4 = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        if (EDGE_G) g4 = gv[qi];
        const unsigned off[4] = {o.x & 0xffffu, o.x >> 16, o.y & 0xffffu, o.y >> 16};
        const float2 gg[2] = {make_float2(g4.x, g4.y), make_float2(g4.z, g4.w)};
        if (INFOLI_KAHAN_BLOCK) {
          // the quad's two terms per accumulator are summed first (one
          // rounding, which the Kahan step after it captures), then
          // Kahan-added: 6 paired instructions per quad instead of 8
          float2 nt[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float2 x = make_float2(*reinterpret_cast<const float*>(sm + off[2 * h]),
                                         *reinterpret_cast<const float*>(sm + off[2 * h + 1]));
            const float2 nv = __fadd2_rn(x, nvc2);  // -V, scaled by kVScale
            const float2 sq = __fmul2_rn(nv, nv);
            const float2 e = make_float2(ex2_approx(-sq.x), ex2_approx(-sq.y));
            float2 f = __ffma2_rn(c08, e, c02);
            if (EDGE_G) f = __fmul2_rn(gg[h], f);
            nt[h] = h == 0 ? __fmul2_rn(f, nv) : __ffma2_rn(f, nv, nt[0]);  // -(t0 + t2), -(t1 + t3)
          }
          const float2 ny = __fadd2_rn(nt[1], cmp);     // -(block - c)
          const float2 ns = __fadd2_rn(nacc, ny);       // -(acc + y)
          const float2 dt = __ffma2_rn(nacc, m1, ns);   // ns - nacc
          cmp = __ffma2_rn(dt, m1, ny);                 // (s - acc) - y
          nacc = ns;
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float2 x = make_float2(*reinterpret_cast<const float*>(sm + off[2 * h]),
                                         *reinterpret_cast<const float*>(sm + off[2 * h + 1]));
            const float2 nv = __fadd2_rn(x, nvc2);  // -V, scaled by kVScale
            const float2 sq = __fmul2_rn(nv, nv);
            const float2 e = make_float2(ex2_approx(-sq.x), ex2_approx(-sq.y));
            float2 f = __ffma2_rn(c08, e, c02);
            if (EDGE_G) f = __fmul2_rn(gg[h], f);
            const float2 ny = __ffma2_rn(f, nv, cmp);      // -(term - c)
            const float2 ns = __fadd2_rn(nacc, ny);        // -(acc + y)
            const float2 dt = __ffma2_rn(nacc, m1, ns);    // ns - nacc
            cmp = __ffma2_rn(dt, m1, ny);                  // ny - (ns - nacc) = (s - acc) - y
            nacc = ns;
          }
        }
      }
      // TwoSum of the two accumulators (values un-negated)
      const float a0 = -nacc.x, a1 = -nacc.y;
      const float sum = a0 + a1;
      const float bb = sum - a0;
      const float err = (a0 - (sum - bb)) + (a1 - bb);  // a0 + a1 = sum + err exactly
      part[d.x] = sum;
      partc[d.x] = (cmp.x + cmp.y) - err;
    }
  }
}

// Phase A for one staged tile: warp w reduces chunks cb+w, cb+w+nwarps, ...
// Each lane takes edges lane, lane+32, ... of the chunk (in unrolled,
// predicated blocks of kChunkEdges; chunks of dense rows are longer, so a
// CTA's partial-sum slots fit in shared memory); a shuffle tree sums the
// lanes; lane 0 writes the chunk's slot.
template <bool KAHAN, bool EDGE_G>
__device__ __forceinline__ void couple_tile(const ChunkDesc* chunks, const uint16_t* edges, const float* edge_g,
                                            int cb, int ce, int edge0, const float* buf, const float* sVd,
                                            float* part, float* partc, int warp, int nwarps, int lane) {
  for (int ci = cb + warp; ci < ce; ci += nwarps) {
    const ChunkDesc c = chunks[ci];
    const float vc = sVd[c.recv];
    const int eb = c.edge_begin - edge0;
    float acc = 0.0f, comp = 0.0f;
    for (int u0 = 0; u0 < c.count; u0 += kChunkEdges) {
#pragma unroll
    for (int q = 0; q < kChunkEdges / 32; ++q) {
      const int u = u0 + lane + 32 * q;
      if (u < c.count) {
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
}

// BLOCK threads per CTA, one CTA per SM: 1024 threads get 64 registers each,
// 512 threads 128 (fewer warps, no spills).
template <int BLOCK, bool KAHAN, bool EDGE_G, bool LL, int NB>
__global__ void __launch_bounds__(BLOCK, 1) step_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  __shared__ unsigned long long s_prof[6];
  const SmemShape shp = a.shape;
  const SmemLayout L = smem_layout(shp);
  float* tbuf = reinterpret_cast<float*>(smem_raw + L.tiles);
  // per-cell arrays: V_dend, V_soma, V_axon, then the nine unit currents
  float* sV = reinterpret_cast<float*>(smem_raw + L.vown);
  const int cap = shp.cells_cap;
  float* sVd = sV;
  float* sVs = sV + cap;
  float* sVa = sV + 2 * cap;
  float* sI = sV + 3 * cap;  // current k of cell r at sI[k * cap + r]
  float* sVq = sV + kScaledVArray * cap;  // stamped plans: V_dend x kVScale
  float* part = reinterpret_cast<float*>(smem_raw + L.part);
  float* partc = reinterpret_cast<float*>(smem_raw + L.partc);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + L.mbar);

  const CtaWork w = a.cta[blockIdx.x];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const bool owner = tid < w.n_cells;  // voltage thread of cell w.cell_begin + tid
  const int cell = w.cell_begin + tid;  // plan cell id (exchange words, plan tables)
  // the caller's id of the cell (state, inputs, traces); plans relabel only
  // stamped exchanges, whose V_dend words are the vll arrays
  const int ocell = (a.perm && owner) ? a.perm[cell] : cell;
  const long long np = a.n_pad;
  const int tile_cap = shp.tile_cap;
  const int nbuf = shp.nbuf;

  // ---- gate units: warp w works on cell group w / U (32 cells) and runs
  // the units u with u % U == w % U; U is the largest of 8, 4, 2, 1 whose
  // groups x U fit in the CTA's warps.  Warp-uniform, so no divergence.
  const int ngroups = (w.n_cells + 31) >> 5;
  int U = kUnits;
  while (U > 1 && ngroups * U > nwarps) U >>= 1;
  const bool unit_warp = warp < ngroups * U;
  const int ucell_l = (warp / U) * 32 + lane;  // local cell of this unit lane
  const bool unit_lane = unit_warp && ucell_l < w.n_cells;
  unsigned umask = 0;
  for (int u = warp % U; u < kUnits; u += U) umask |= 1u << u;
  // stamped mode: threads from poll_first on gather the neighbours' words --
  // the warps left over by the gate units when they can take every word in
  // one batch of loads (they poll while the units compute), else every thread
  // after its units
  PollWindow pw{};
  int poll_first = 0;
  if (LL) {
    pw.probes = a.probes + w.probe_begin;
    pw.n_probes = w.n_probes;
    pw.tile_words = w.n_tiles;  // stamped plans: window words (gcol[tile_begin ..])
    pw.total = pw.tile_words + pw.n_probes;
    const int pollers = (int)blockDim.x - ngroups * U * 32;
    if (ngroups * U < nwarps && pollers * NB >= pw.total) poll_first = ngroups * U * 32;
  }
  // (Issuing the first poll batch before the gate units was measured slower:
  // the outstanding loads delay the units' shared-memory traffic.)

  // ---- static work: either resident in shared memory or read from global.
  // Indices below are relative to the CTA's first chunk / edge.
  const TileDesc* tiles = LL ? nullptr : a.tiles + w.tile_begin;  // stamped: tile_begin indexes gcol
  const ChunkDesc* chunks = a.chunks;
  const uint16_t* edges = a.edges;
  const float* edge_g = a.edge_g;
  int chunk0 = 0, edge0 = 0;
  if (LL) {
    // stamped plans: window sender ids (in the descriptor area) + packed
    // lane-chunk groups, copied once per launch
    int* s_w = reinterpret_cast<int*>(smem_raw + L.tdesc);
    int2* s_d = reinterpret_cast<int2*>(smem_raw + L.chunks);
    uint2* s_e = reinterpret_cast<uint2*>(smem_raw + L.edges);
    float4* s_g = reinterpret_cast<float4*>(smem_raw + L.eg);
    for (int i = tid; i < w.n_tiles; i += blockDim.x) s_w[i] = a.gcol[w.tile_begin + i];
    const int nd = w.n_groups * 32;
    for (int i = tid; i < nd; i += blockDim.x) s_d[i] = a.gdesc[(size_t)w.group_begin * 32 + i];
    const int nq = w.n_groups * (kGroupEntries / 4);  // 8-byte quads
    const uint2* ge = reinterpret_cast<const uint2*>(a.edges) + (size_t)w.group_begin * (kGroupEntries / 4);
    for (int i = tid; i < nq; i += blockDim.x) s_e[i] = ge[i];
    if (EDGE_G) {
      const float4* gg = reinterpret_cast<const float4*>(a.edge_g) + (size_t)w.group_begin * (kGroupEntries / 4);
      for (int i = tid; i < nq; i += blockDim.x) s_g[i] = gg[i];
    }
    pw.cells = s_w;
  } else if (w.n_tiles > 0) {
    chunk0 = tiles[0].chunk_begin;
    const int chunk1 = tiles[w.n_tiles - 1].chunk_end;
    edge0 = chunk1 > chunk0 ? a.chunks[chunk0].edge_begin : 0;
    if (shp.res_chunks > 0) {
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

  // stamped plans read each receiver's partial slots four at a time: the gaps
  // between receivers' slot blocks must hold zeros (nothing writes them)
  if (LL)
    for (int i = tid; i < shp.max_slots; i += blockDim.x) {
      part[i] = 0.0f;
      if (KAHAN) partc[i] = 0.0f;
    }
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }

  // gate state of the owned cells lives in shared memory for the launch:
  // field f of local cell r at sG[f * cap + r] (f = DevField), Ca2+ in sCa[r]
  float* sG = reinterpret_cast<float*>(smem_raw + L.gates);
  double* sCa = reinterpret_cast<double*>(smem_raw + L.gca);
  if (owner) {
    const float* st = a.st;
    for (int f = F_Q; f < F_COUNT; ++f) sG[f * cap + tid] = st[f * np + ocell];
    sCa[tid] = a.ca[ocell];
  }
  // voltage threads hold the per-cell constants of the voltage step
  int2 slots = make_int2(0, 0);
  float gscale = a.g_uniform;
  float my_amp = 0.0f;
  int my_onset = 0, my_off = 0;
  if (owner) {
    sVd[tid] = a.vd[a.step0 & 1][ocell];
    if (LL) sVq[tid] = sVd[tid] * kVScale;
    sVs[tid] = a.st[F_VS * np + ocell];
    sVa[tid] = a.st[F_VA * np + ocell];
    slots = a.cell_slots[cell];
    if (a.cell_g) gscale = a.cell_g[ocell];
    if (a.stim_kind == STIM_CELL) {
      my_amp = a.cell_amp[ocell];
      my_onset = a.cell_onset[ocell];
    }
    if (a.cell_step_off) my_off = a.cell_step_off[ocell];
  }
  const VoltCoef vk = volt_coef(a.P);
  const bool prof = a.prof != nullptr && tid == 0;
  if (prof) s_prof[0] = s_prof[1] = s_prof[2] = s_prof[3] = s_prof[4] = s_prof[5] = 0;
  __syncthreads();

  // phase timers count SM cycles; the launch's global-timer span calibrates them
  const uint64_t ns_begin = prof ? globaltimer_ns() : 0;
  const uint64_t cy_begin = prof ? clock64() : 0;
  uint64_t t_step = cy_begin;
  unsigned nload = 0;  // bulk tile loads issued so far (same value in every thread)
  int row = 0;
  unsigned bar_target = 0;
  if (LL && owner) {
    // publish V^step0 with its stamp (the host cleared both slots before launch)
    if ((int)blockIdx.x != a.stall_cta)
      st_relaxed_gpu_u64(a.vll[a.step0 & 1] + cell, pack_stamp(sVd[tid], (unsigned)a.step0));
  }
  TraceClock tclock(a.trace_every, a.step0);
  for (int t = 0; t < a.n_steps; ++t) {
    const int step = a.step0 + t;
    const bool trace_now = tclock.take();
    const float* vcur = a.vd[step & 1];
    uint64_t t_ready = 0;

    // ---------------- first tile in flight while the gate units run
    if (!LL && w.n_tiles > 0 && tid == 0) {
      fence_proxy_async_global();
      fence_proxy_async_smem();
      issue_tile(a, vcur, tiles[0], tbuf + (nload % nbuf) * tile_cap, &mbar[nload % nbuf]);
    }

    // ---------------- first poll batch in flight during the gate units
    // (every thread polls: no spare warps)
    PollLean<(kPollEarly > 0 ? kPollEarly : 1)> early;
    const bool poll_early = LL && !KAHAN && kPollEarly > 0 && poll_first == 0;
    if (poll_early) poll_issue_lean(a, a.vll[step & 1], pw, tid, (int)blockDim.x, tbuf, shp.dup_words, early);

    // ---------------- gate units (old voltages only)
    if (unit_lane) {
      Volts v;
      v.Vd = sVd[ucell_l];
      v.Vs = sVs[ucell_l];
      v.Va = sVa[ucell_l];
      Currents cur;
      Gates gs = load_gates(sG, sCa, cap, ucell_l, umask);
      run_units(a.P, umask, v, gs, cur);
      store_gates(sG, sCa, cap, ucell_l, umask, gs);
      if (umask & 0x01u) sI[0 * cap + ucell_l] = cur.I_h;
      if (umask & 0x02u) {
        sI[1 * cap + ucell_l] = cur.I_CaH;
        sI[2 * cap + ucell_l] = cur.I_K_Ca;
      }
      if (umask & 0x04u) sI[3 * cap + ucell_l] = cur.I_CaL;
      if (umask & 0x08u) sI[4 * cap + ucell_l] = cur.I_Na_s;
      if (umask & 0x10u) sI[5 * cap + ucell_l] = cur.I_Kdr_s;
      if (umask & 0x20u) sI[6 * cap + ucell_l] = cur.I_K_s;
      if (umask & 0x40u) sI[7 * cap + ucell_l] = cur.I_Na_a;
      if (umask & 0x80u) sI[8 * cap + ucell_l] = cur.I_K_a;
    }
    const uint64_t t_units = prof ? clock64() : 0;

    // ---------------- phase A: gap-junction coupling
    if (LL) {
      // stamped exchange: gather the whole window (and the progress probes)
      // once the words carry this step's stamp, then reduce all chunks.  The
      // polling threads are the warps without gate units when there are any
      // (they poll while the units compute), else every thread after its units.
      if (tid >= poll_first) {
        const unsigned long long* vsrc = a.vll[step & 1];
        const int pt = tid - poll_first, npt = blockDim.x - poll_first;
        uint64_t pt0 = 0;
        bool ok = true;
        int base0 = pt;
        if (poll_early) {
          ok = poll_finish_lean(a, vsrc, pw, pt, npt, tbuf, shp.dup_words, (unsigned)step, early, pt0);
          base0 = pt + kPollEarly * npt;
        }
        PollBatchT<NB> pb;
        for (int base = base0; ok && base < pw.total; base += NB * npt) {
          poll_issue(a, vsrc, pw, base, npt, tbuf, shp.dup_words, pb);
          ok = poll_finish<NB, KAHAN && NB <= kPollBatchSmall>(a, vsrc, tbuf, shp.dup_words, (unsigned)step, pb, pt0);
        }
        if (!ok) s_abort = 1;
      }
      __syncthreads();
      if (s_abort) break;
      if (prof) t_ready = clock64();
      couple_packed<KAHAN, EDGE_G>(smem_raw, L, w.n_groups, sVq, part, partc, warp, nwarps, lane);
      __syncthreads();
    } else if (w.n_tiles > 0) {
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
        if (prof && j == 0) t_ready = clock64();
        couple_tile<KAHAN, EDGE_G>(chunks, edges, edge_g, td.chunk_begin - chunk0, td.chunk_end - chunk0, edge0,
                                   buf, sVd, part, partc, warp, nwarps, lane);
        __syncthreads();
      }
      nload += w.n_tiles;
    } else {
      if (prof) t_ready = clock64();
      __syncthreads();
    }
    const uint64_t t_coupled = prof ? clock64() : 0;

    // ---------------- phase B: voltage step, one thread per owned cell
    if (owner) {
      float ic;
      if (KAHAN && LL) {
        // stamped plans: float4 reads of the partial sums and their
        // compensations (slot blocks 16-byte aligned, zero gaps).  The partials
        // are added in slot order with an error-free TwoSum per addition, so
        // the dependent chain is one add per slot; the rounding errors and the
        // lanes' compensations are summed beside it and applied once.
        float s = 0.0f, e = 0.0f, c = 0.0f;
        const float4* p4 = reinterpret_cast<const float4*>(part + slots.x);
        const float4* c4 = reinterpret_cast<const float4*>(partc + slots.x);
        const int nq = (slots.y + 3) >> 2;
        for (int q = 0; q < nq; ++q) {
          const float4 p = p4[q];
          const float4 cc = c4[q];
          c += (cc.x + cc.y) + (cc.z + cc.w);
          const float pv[4] = {p.x, p.y, p.z, p.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float t = s + pv[j];
            const float bp = t - s;
            e += (s - (t - bp)) + (pv[j] - bp);
            s = t;
          }
        }
        ic = s + (e - c);
      } else if (KAHAN) {
        float s = 0.0f, cmp = 0.0f;
        for (int q = 0; q < slots.y; ++q) {
          const float y = part[slots.x + q] - (partc[slots.x + q] + cmp);
          const float tt = s + y;
          cmp = (tt - s) - y;
          s = tt;
        }
        ic = s;
      } else if (LL) {
        // stamped plans: a receiver's slots start on a 16-byte boundary and the
        // gaps after them hold zeros, so read them as float4 (slot order kept)
        ic = 0.0f;
        const float4* p4 = reinterpret_cast<const float4*>(part + slots.x);
        const int nq = (slots.y + 3) >> 2;
        for (int q = 0; q < nq; ++q) {
          const float4 p = p4[q];
          ic += p.x;
          ic += p.y;
          ic += p.z;
          ic += p.w;
        }
      } else {
        // in slot (= sender) order; four loads in flight at a time
        ic = 0.0f;
        const float* ps = part + slots.x;
        int q = 0;
        for (; q + 4 <= slots.y; q += 4) {
          const float p0 = ps[q], p1 = ps[q + 1], p2 = ps[q + 2], p3 = ps[q + 3];
          ic += p0;
          ic += p1;
          ic += p2;
          ic += p3;
        }
        for (; q < slots.y; ++q) ic += ps[q];
      }
      if (LL) ic *= kInvVScale;  // stamped partial sums are in scaled units
      if (!EDGE_G) ic *= gscale;
      const int ls = step + my_off;
      float iapp;
      if (a.stim_kind == STIM_PULSE)
        iapp = (ls >= a.stim_start && ls < a.stim_end) ? a.stim_amp : 0.0f;
      else if (a.stim_kind == STIM_CELL)
        iapp = (ls >= my_onset && ls < my_onset + a.stim_dur) ? my_amp : 0.0f;
      else
        iapp = a.stim_table[(size_t)t * np + ocell];
      Currents cur;
      cur.I_h = sI[0 * cap + tid];
      cur.I_CaH = sI[1 * cap + tid];
      cur.I_K_Ca = sI[2 * cap + tid];
      cur.I_CaL = sI[3 * cap + tid];
      cur.I_Na_s = sI[4 * cap + tid];
      cur.I_Kdr_s = sI[5 * cap + tid];
      cur.I_K_s = sI[6 * cap + tid];
      cur.I_Na_a = sI[7 * cap + tid];
      cur.I_K_a = sI[8 * cap + tid];
      Volts v;
      v.Vd = sVd[tid];
      v.Vs = sVs[tid];
      v.Va = sVa[tid];
      voltage_step(a.P, vk, v, cur, ic, iapp);
      if (!LL)
        a.vd[(step + 1) & 1][cell] = v.Vd;
      else if ((int)blockIdx.x != a.stall_cta)
        st_relaxed_gpu_u64(a.vll[(step + 1) & 1] + cell, pack_stamp(v.Vd, (unsigned)(step + 1)));
      sVd[tid] = v.Vd;
      if (LL) sVq[tid] = v.Vd * kVScale;
      sVs[tid] = v.Vs;
      sVa[tid] = v.Va;
      if (trace_now) {
        float* tr = a.trace + (size_t)row * a.trace_nq * np + ocell;
        int qi = 0;
        if (a.trace_mask & TRACE_AXON) tr[(qi++) * np] = v.Va;
        if (a.trace_mask & TRACE_SOMA) tr[(qi++) * np] = v.Vs;
        if (a.trace_mask & TRACE_DEND) tr[(qi++) * np] = v.Vd;
      }
    }
    if (trace_now) ++row;

    if (LL) {
      uint64_t t_arrive = prof ? clock64() : 0;
      __syncthreads();  // new voltages / free tile buffers before the next step
      if (prof) {
        const uint64_t t_done = clock64();
        s_prof[0] += t_ready - t_units;
        s_prof[5] += t_units - t_step;
        s_prof[1] += t_coupled - t_ready;
        s_prof[2] += t_arrive - t_coupled;
        s_prof[3] += t_done - t_arrive;
        s_prof[4] += 1;
        t_step = t_done;
      }
    } else if (t + 1 < a.n_steps) {
      bar_target += gridDim.x;
      uint64_t t_arrive = 0;
      const bool ok = grid_sync(a, bar_target, &s_abort, prof ? &t_arrive : nullptr);
      if (prof) {
        const uint64_t t_done = clock64();
        s_prof[0] += t_ready - t_units;
        s_prof[5] += t_units - t_step;
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
    atomicAdd(pr + PROF_UNITS, s_prof[5]);
    atomicAdd(pr + PROF_SPAN_NS, (unsigned long long)(globaltimer_ns() - ns_begin));
    atomicAdd(pr + PROF_SPAN_CYCLES, (unsigned long long)(clock64() - cy_begin));
  }
  __syncthreads();

  if (owner) {
    float* st = a.st;
    for (int f = F_Q; f < F_COUNT; ++f) st[f * np + ocell] = sG[f * cap + tid];
    a.ca[ocell] = sCa[tid];
    if (LL) a.vd[(a.step0 + a.n_steps) & 1][ocell] = sVd[tid];
    st[F_VS * np + ocell] = sVs[tid];
    st[F_VA * np + ocell] = sVa[tid];
  }
}

// Gather plans (sparse networks whose sender windows do not fit in shared
// memory): one thread per receiver, state in registers, edges of a CTA's
// receivers stored column by column (entry j of local receiver t at
// base + j * n_cells + t, rows padded to the CTA's longest row with the
// receiver itself, which adds exactly 0), so each load instruction of a warp
// reads 32 consecutive entries; the senders' V_dend is read from the global
// double buffer through L2.  One grid barrier per step.  Senders are summed in
// the receiver's CSR order.
// Gate state of the gather kernel in shared memory (15 floats + FP64 Ca2+ per
// cell), so the coupling loop has the registers for many loads in flight.
constexpr int kGatherGateFloats = 15;
constexpr int kGatherGroup = 8;  // V_dend loads in flight per thread

__device__ __forceinline__ void gather_store_gates(float* sg, double* sca, int blk, int t, const Gates& g) {
  const float f[kGatherGateFloats] = {g.q, g.r, g.s, g.ICaH, g.gCaL, g.k, g.l, g.m,
                                      g.h, g.n, g.p, g.xs, g.ma, g.ha, g.xa};
#pragma unroll
  for (int i = 0; i < kGatherGateFloats; ++i) sg[i * blk + t] = f[i];
  sca[t] = g.Ca;
}

__device__ __forceinline__ Gates gather_load_gates(const float* sg, const double* sca, int blk, int t) {
  Gates g;
  g.q = sg[0 * blk + t];
  g.r = sg[1 * blk + t];
  g.s = sg[2 * blk + t];
  g.ICaH = sg[3 * blk + t];
  g.gCaL = sg[4 * blk + t];
  g.k = sg[5 * blk + t];
  g.l = sg[6 * blk + t];
  g.m = sg[7 * blk + t];
  g.h = sg[8 * blk + t];
  g.n = sg[9 * blk + t];
  g.p = sg[10 * blk + t];
  g.xs = sg[11 * blk + t];
  g.ma = sg[12 * blk + t];
  g.ha = sg[13 * blk + t];
  g.xa = sg[14 * blk + t];
  g.Ca = sca[t];
  return g;
}

size_t gather_smem_bytes(int block) { return (size_t)block * (kGatherGateFloats * sizeof(float) + sizeof(double)); }

// Gather plans (sparse networks whose sender windows do not fit in shared
// memory): one thread per receiver, voltages in registers and gate state in
// shared memory; edges of a CTA's receivers stored column by column (entry j
// of local receiver t at base + j * n_cells + t, rows padded to the CTA's
// longest row with the receiver itself, which adds exactly 0), so each load
// instruction of a warp reads 32 consecutive entries; the senders' V_dend is
// read from the global double buffer through L2, kGatherGroup loads in flight
// per thread with the next group's sender ids already loaded.  One grid
// barrier per step.  Senders are summed in the receiver's CSR order.
template <int BLOCK, bool KAHAN, bool EDGE_G>
__global__ void __launch_bounds__(BLOCK, 1) gather_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sCa = reinterpret_cast<double*>(smem_raw);
  float* sGt = reinterpret_cast<float*>(smem_raw + sizeof(double) * BLOCK);
  __shared__ int s_abort;
  const CtaWork w = a.cta[blockIdx.x];
  const int tid = threadIdx.x;
  const bool owner = tid < w.n_cells;
  const int cell = w.cell_begin + tid;
  const long long np = a.n_pad;
  if (tid == 0) s_abort = 0;
  Volts v{};
  float my_amp = 0.0f;
  int my_onset = 0, my_off = 0;
  if (owner) {
    const float* st = a.st;
    v.Vd = a.vd[a.step0 & 1][cell];
    v.Vs = st[F_VS * np + cell];
    v.Va = st[F_VA * np + cell];
    Gates g;
    g.q = st[F_Q * np + cell];
    g.r = st[F_R * np + cell];
    g.s = st[F_S * np + cell];
    g.Ca = a.ca[cell];
    g.ICaH = st[F_ICAH * np + cell];
    g.gCaL = st[F_GCAL * np + cell];
    g.k = st[F_K * np + cell];
    g.l = st[F_L * np + cell];
    g.m = st[F_M * np + cell];
    g.h = st[F_H * np + cell];
    g.n = st[F_N * np + cell];
    g.p = st[F_P * np + cell];
    g.xs = st[F_XS * np + cell];
    g.ma = st[F_MA * np + cell];
    g.ha = st[F_HA * np + cell];
    g.xa = st[F_XA * np + cell];
    gather_store_gates(sGt, sCa, BLOCK, tid, g);
    if (a.stim_kind == STIM_CELL) {
      my_amp = a.cell_amp[cell];
      my_onset = a.cell_onset[cell];
    }
    if (a.cell_step_off) my_off = a.cell_step_off[cell];
  }
  const int deg = w.pad0;
  const int stride = w.n_cells;
  const int* __restrict__ ecol = a.gcol + (size_t)w.slot_begin + tid;
  const float* __restrict__ eg = EDGE_G ? a.edge_g + (size_t)w.slot_begin + tid : nullptr;
  const VoltCoef vk = volt_coef(a.P);
  unsigned bar_target = 0;
  int row = 0;
  __syncthreads();
  TraceClock tclock(a.trace_every, a.step0);
  for (int t = 0; t < a.n_steps; ++t) {
    const int step = a.step0 + t;
    const bool trace_now = tclock.take();
    if (owner) {
      const float* __restrict__ vcur = a.vd[step & 1];
      const float vc = v.Vd;
      float acc = 0.0f, comp = 0.0f;
      int nidx[kGatherGroup];
#pragma unroll
      for (int u = 0; u < kGatherGroup; ++u) nidx[u] = (u < deg) ? __ldg(ecol + (size_t)u * stride) : cell;
      for (int j = 0; j < deg; j += kGatherGroup) {
        float vs[kGatherGroup], gg[kGatherGroup];
#pragma unroll
        for (int u = 0; u < kGatherGroup; ++u) {
          vs[u] = __ldcg(vcur + nidx[u]);  // past the row end: the receiver itself
          gg[u] = (EDGE_G && j + u < deg) ? __ldg(eg + (size_t)(j + u) * stride) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kGatherGroup; ++u) {
          const int jn = j + kGatherGroup + u;
          nidx[u] = (jn < deg) ? __ldg(ecol + (size_t)jn * stride) : cell;
        }
#pragma unroll
        for (int u = 0; u < kGatherGroup; ++u) {
          const float V = vc - vs[u];
          const float f = fmaf(0.8f, ex2_approx((V * V) * kNegLog2eOver100), 0.2f);
          const float term = EDGE_G ? (gg[u] * f) * V : f * V;
          if (KAHAN) {
            const float y = term - comp;
            const float s2 = acc + y;
            comp = (s2 - acc) - y;
            acc = s2;
          } else {
            acc += term;
          }
        }
      }
      const float ic = EDGE_G ? acc : acc * a.g_uniform;
      const int ls = step + my_off;
      float iapp;
      if (a.stim_kind == STIM_PULSE)
        iapp = (ls >= a.stim_start && ls < a.stim_end) ? a.stim_amp : 0.0f;
      else if (a.stim_kind == STIM_CELL)
        iapp = (ls >= my_onset && ls < my_onset + a.stim_dur) ? my_amp : 0.0f;
      else
        iapp = a.stim_table[(size_t)t * np + cell];
      Gates g = gather_load_gates(sGt, sCa, BLOCK, tid);
      Currents cur;
      run_units(a.P, 0xffu, v, g, cur);
      voltage_step(a.P, vk, v, cur, ic, iapp);
      gather_store_gates(sGt, sCa, BLOCK, tid, g);
      a.vd[(step + 1) & 1][cell] = v.Vd;
      if (trace_now) {
        float* tr = a.trace + (size_t)row * a.trace_nq * np + cell;
        int qi = 0;
        if (a.trace_mask & TRACE_AXON) tr[(qi++) * np] = v.Va;
        if (a.trace_mask & TRACE_SOMA) tr[(qi++) * np] = v.Vs;
        if (a.trace_mask & TRACE_DEND) tr[(qi++) * np] = v.Vd;
      }
    }
    if (trace_now) ++row;
    if (t + 1 < a.n_steps) {
      bar_target += gridDim.x;
      if (!grid_sync(a, bar_target, &s_abort, nullptr)) break;
    }
  }
  if (owner) {
    const Gates g = gather_load_gates(sGt, sCa, BLOCK, tid);
    float* st = a.st;
    st[F_VS * np + cell] = v.Vs;
    st[F_VA * np + cell] = v.Va;
    st[F_Q * np + cell] = g.q;
    st[F_R * np + cell] = g.r;
    st[F_S * np + cell] = g.s;
    a.ca[cell] = g.Ca;
    st[F_ICAH * np + cell] = g.ICaH;
    st[F_GCAL * np + cell] = g.gCaL;
    st[F_K * np + cell] = g.k;
    st[F_L * np + cell] = g.l;
    st[F_M * np + cell] = g.m;
    st[F_H * np + cell] = g.h;
    st[F_N * np + cell] = g.n;
    st[F_P * np + cell] = g.p;
    st[F_XS * np + cell] = g.xs;
    st[F_MA * np + cell] = g.ma;
    st[F_HA * np + cell] = g.ha;
    st[F_XA * np + cell] = g.xa;
  }
}

// Tiled gather plans: one thread per receiver with its state in registers;
// each step the CTA's tiles of V_dend are staged into shared memory by bulk
// async copies (two buffers when there are several tiles: the next tile's
// copy overlaps this tile's gathers) and every receiver walks its senders in
// the tile (16-bit offsets, column by column, its own count).  One grid
// barrier per step; senders are summed tile by tile in ascending order.
template <int BLOCK, bool KAHAN, bool EDGE_G>
__global__ void __launch_bounds__(BLOCK, 1) tgather_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  float* tbuf = reinterpret_cast<float*>(smem_raw);
  const int tile_cap = a.shape.tile_cap, nbuf = a.shape.nbuf;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(
      smem_raw + (((size_t)nbuf * (size_t)tile_cap * sizeof(float) + 15) & ~(size_t)15));
  const CtaWork w = a.cta[blockIdx.x];
  const TileDesc* tiles = a.tiles + w.tile_begin;
  const int tid = threadIdx.x;
  const bool owner = tid < w.n_cells;
  const int cell = w.cell_begin + tid;
  const long long np = a.n_pad;
  const int nc = w.n_cells;
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  Volts v{};
  Gates g{};
  float my_amp = 0.0f;
  int my_onset = 0, my_off = 0;
  if (owner) {
    const float* st = a.st;
    v.Vd = a.vd[a.step0 & 1][cell];
    v.Vs = st[F_VS * np + cell];
    v.Va = st[F_VA * np + cell];
    g.q = st[F_Q * np + cell];
    g.r = st[F_R * np + cell];
    g.s = st[F_S * np + cell];
    g.Ca = a.ca[cell];
    g.ICaH = st[F_ICAH * np + cell];
    g.gCaL = st[F_GCAL * np + cell];
    g.k = st[F_K * np + cell];
    g.l = st[F_L * np + cell];
    g.m = st[F_M * np + cell];
    g.h = st[F_H * np + cell];
    g.n = st[F_N * np + cell];
    g.p = st[F_P * np + cell];
    g.xs = st[F_XS * np + cell];
    g.ma = st[F_MA * np + cell];
    g.ha = st[F_HA * np + cell];
    g.xa = st[F_XA * np + cell];
    if (a.stim_kind == STIM_CELL) {
      my_amp = a.cell_amp[cell];
      my_onset = a.cell_onset[cell];
    }
    if (a.cell_step_off) my_off = a.cell_step_off[cell];
  }
  const int* __restrict__ counts = a.gcol + (size_t)w.slot_begin + tid;
  const VoltCoef vk = volt_coef(a.P);
  unsigned bar_target = 0, nload = 0;
  int row = 0;
  __syncthreads();
  TraceClock tclock(a.trace_every, a.step0);
  for (int t = 0; t < a.n_steps; ++t) {
    const int step = a.step0 + t;
    const bool trace_now = tclock.take();
    const float* vcur = a.vd[step & 1];
    float acc = 0.0f, comp = 0.0f;
    if (w.n_tiles > 0 && tid == 0) {
      fence_proxy_async_global();
      fence_proxy_async_smem();
      issue_tile(a, vcur, tiles[0], tbuf + (nload % nbuf) * tile_cap, &mbar[nload % nbuf]);
    }
    for (int j = 0; j < w.n_tiles; ++j) {
      const TileDesc td = tiles[j];
      const unsigned k = nload + j;
      const int b = (int)(k % (unsigned)nbuf);
      const float* buf = tbuf + b * tile_cap;
      if (tid == 0 && j > 0 && nbuf == 1) {
        fence_proxy_async_smem();
        issue_tile(a, vcur, td, tbuf, &mbar[0]);
      }
      if (tid == 0 && j + 1 < w.n_tiles && nbuf == 2) {
        fence_proxy_async_smem();
        const int b1 = (int)((k + 1) & 1u);
        issue_tile(a, vcur, tiles[j + 1], tbuf + b1 * tile_cap, &mbar[b1]);
      }
      const int cnt = owner ? __ldg(counts + (size_t)j * nc) : 0;
      if (!wait_tile(a, &mbar[b], (k / (unsigned)nbuf) & 1u)) s_abort = 1;
      if (owner) {
        const uint16_t* __restrict__ ent = a.edges + (size_t)td.chunk_begin + tid;
        const float* __restrict__ eg = EDGE_G ? a.edge_g + (size_t)td.chunk_begin + tid : nullptr;
        const float vc = v.Vd;
#pragma unroll 4
        for (int q = 0; q < cnt; ++q) {
          const float V = vc - buf[__ldg(ent + (size_t)q * nc)];
          const float f = fmaf(0.8f, ex2_approx((V * V) * kNegLog2eOver100), 0.2f);
          const float term = EDGE_G ? (__ldg(eg + (size_t)q * nc) * f) * V : f * V;
          if (KAHAN) {
            const float y = term - comp;
            const float s2 = acc + y;
            comp = (s2 - acc) - y;
            acc = s2;
          } else {
            acc += term;
          }
        }
      }
      __syncthreads();  // every thread is done with this buffer before it is refilled
    }
    nload += w.n_tiles;
    if (s_abort) break;
    if (owner) {
      const float ic = EDGE_G ? acc : acc * a.g_uniform;
      const int ls = step + my_off;
      float iapp;
      if (a.stim_kind == STIM_PULSE)
        iapp = (ls >= a.stim_start && ls < a.stim_end) ? a.stim_amp : 0.0f;
      else if (a.stim_kind == STIM_CELL)
        iapp = (ls >= my_onset && ls < my_onset + a.stim_dur) ? my_amp : 0.0f;
      else
        iapp = a.stim_table[(size_t)t * np + cell];
      Currents cur;
      run_units(a.P, 0xffu, v, g, cur);
      voltage_step(a.P, vk, v, cur, ic, iapp);
      a.vd[(step + 1) & 1][cell] = v.Vd;
      if (trace_now) {
        float* tr = a.trace + (size_t)row * a.trace_nq * np + cell;
        int qi = 0;
        if (a.trace_mask & TRACE_AXON) tr[(qi++) * np] = v.Va;
        if (a.trace_mask & TRACE_SOMA) tr[(qi++) * np] = v.Vs;
        if (a.trace_mask & TRACE_DEND) tr[(qi++) * np] = v.Vd;
      }
    }
    if (trace_now) ++row;
    if (t + 1 < a.n_steps) {
      bar_target += gridDim.x;
      if (!grid_sync(a, bar_target, &s_abort, nullptr)) break;
    }
  }
  if (owner) {
    float* st = a.st;
    st[F_VS * np + cell] = v.Vs;
    st[F_VA * np + cell] = v.Va;
    st[F_Q * np + cell] = g.q;
    st[F_R * np + cell] = g.r;
    st[F_S * np + cell] = g.s;
    a.ca[cell] = g.Ca;
    st[F_ICAH * np + cell] = g.ICaH;
    st[F_GCAL * np + cell] = g.gCaL;
    st[F_K * np + cell] = g.k;
    st[F_L * np + cell] = g.l;
    st[F_M * np + cell] = g.m;
    st[F_H * np + cell] = g.h;
    st[F_N * np + cell] = g.n;
    st[F_P * np + cell] = g.p;
    st[F_XS * np + cell] = g.xs;
    st[F_MA * np + cell] = g.ma;
    st[F_HA * np + cell] = g.ha;
    st[F_XA * np + cell] = g.xa;
  }
}

// Bitmask plans (one conductance, dense rows, windows larger than shared
// memory).  Each CTA stages the whole V_dend array tile by tile like the tiled
// gather kernel; threads are (slice, receiver) pairs, `slices` per receiver,
// and a warp (32 receivers of one slice) walks its share of each tile's
// 32-sender columns in lockstep: per column, as many iterations as the fullest
// of its 32 words has bits, each taking every lane's next set bit (leading
// zeros) and reading that sender's V_dend inside the same 32 staged floats
// (no bank conflicts).  Words come from global memory (coalesced: word w of
// local receiver t at base + w * n_cells + t), two columns ahead.  Column sums
// are compensated with KAHAN; the slices' sums are added in slice order by the
// receiver's owner thread, which then runs the cell update.  One grid barrier
// per step.
// Lockstep iterations per trip of the bitmask walk.
#ifndef INFOLI_BITS_UNROLL
#define INFOLI_BITS_UNROLL 2
#endif

// One lockstep iteration: the lane's next set bit of x (leading zeros; 32
// once x is used up, which reads the next column's first float and adds
// nothing), that sender's staged V_dend x kVScale, its term added to col.
__device__ __forceinline__ void bits_take(uint32_t& x, uint32_t vcol, float vc, float& col) {
  const int c = __clz(x);
  const bool live = x != 0u;
  x &= __funnelshift_rc(0x7fffffffu, 0u, (unsigned)c);
  const float V = vc - ld_shared_f32(vcol + 4u * (uint32_t)c);  // scaled by kVScale
  const float f = fmaf(0.8f, ex2_approx(-(V * V)), 0.2f);
  if (live) col = fmaf(f, V, col);
}

template <bool KAHAN>
__device__ __forceinline__ void bits_walk(bool own, const uint32_t* gw, int stride, int cs, int ce, uint32_t vtile,
                                          int c0, float vc, float& acc, float& cmp) {
  if (cs >= ce) return;
  uint32_t nx = 0u, nnx = 0u;
  if (own) {
    nx = __ldg(gw + (size_t)cs * stride);
    nnx = __ldg(gw + (size_t)(cs + 1) * stride);
  }
  for (int w = cs; w < ce; ++w) {
    uint32_t x = nx;
    nx = nnx;
    ld_global_if(nnx, gw + (size_t)(w + 2) * stride, own);  // rows end with two zero words
    const int m = (int)__reduce_max_sync(0xffffffffu, (unsigned)__popc(x));
    const uint32_t vcol = vtile + 128u * (uint32_t)(w - c0);
    float col = 0.0f;
    // INFOLI_BITS_UNROLL iterations per trip (less loop control), then the
    // rest one at a time: the same terms in the same order either way
    int k = 0;
    for (; k + INFOLI_BITS_UNROLL <= m; k += INFOLI_BITS_UNROLL) {
#pragma unroll
      for (int u = 0; u < INFOLI_BITS_UNROLL; ++u) bits_take(x, vcol, vc, col);
    }
#pragma unroll 1
    for (; k < m; ++k) bits_take(x, vcol, vc, col);
    if (KAHAN) {
      const float y = col - cmp;
      const float t2 = acc + y;
      cmp = (t2 - acc) - y;
      acc = t2;
    } else {
      acc += col;
    }
  }
}

template <int BLOCK, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, 1) bits_kernel(const __grid_constant__ StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_abort;
  float* tbuf = reinterpret_cast<float*>(smem_raw);
  const int tile_cap = a.shape.tile_cap, nbuf = a.shape.nbuf;
  const int R = a.shape.cells_cap, S = a.shape.slices;
  const size_t toff = ((size_t)nbuf * (size_t)tile_cap * sizeof(float) + 15) & ~(size_t)15;
  float* part = reinterpret_cast<float*>(smem_raw + toff);  // [S][R] sums, then [S][R] compensations
  float* partc = part + (size_t)S * R;
  float* sVd = partc + (size_t)S * R;                       // [R] V_dend of the CTA's receivers
  uint64_t* mbar = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(sVd + R));
  const CtaWork w = a.cta[blockIdx.x];
  const TileDesc* tiles = a.tiles + w.tile_begin;
  const int tid = threadIdx.x;
  const int slice = tid / R, t = tid % R;
  const int nc = w.n_cells;
  const bool owner = slice == 0 && t < nc;
  const bool walker = slice < S && (t & ~31) < nc;  // warp-uniform
  const bool own = slice < S && t < nc;
  const int cell = w.cell_begin + t;
  const long long np = a.n_pad;
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  Volts v{};
  Gates g{};
  if (owner) {
    const float* st = a.st;
    v.Vd = a.vd[a.step0 & 1][cell];
    v.Vs = st[F_VS * np + cell];
    v.Va = st[F_VA * np + cell];
    g.q = st[F_Q * np + cell];
    g.r = st[F_R * np + cell];
    g.s = st[F_S * np + cell];
    g.Ca = a.ca[cell];
    g.ICaH = st[F_ICAH * np + cell];
    g.gCaL = st[F_GCAL * np + cell];
    g.k = st[F_K * np + cell];
    g.l = st[F_L * np + cell];
    g.m = st[F_M * np + cell];
    g.h = st[F_H * np + cell];
    g.n = st[F_N * np + cell];
    g.p = st[F_P * np + cell];
    g.xs = st[F_XS * np + cell];
    g.ma = st[F_MA * np + cell];
    g.ha = st[F_HA * np + cell];
    g.xa = st[F_XA * np + cell];
  }
  float my_amp = 0.0f;
  int my_onset = 0, my_off = 0;
  if (owner) {
    if (a.stim_kind == STIM_CELL) {
      my_amp = a.cell_amp[cell];
      my_onset = a.cell_onset[cell];
    }
    if (a.cell_step_off) my_off = a.cell_step_off[cell];
  }
  const uint32_t* gw = reinterpret_cast<const uint32_t*>(a.gcol) + (size_t)w.slot_begin + (own ? t : 0);
  const uint32_t tsm = smem_u32(tbuf);
  const VoltCoef vk = volt_coef(a.P);
  unsigned bar_target = 0, nload = 0;
  int row = 0;
  // the staged tiles hold V_dend x kVScale (an edge's exponent is then
  // -(dV')^2, one multiply less per lockstep iteration): seed this launch's
  // first step from the state, once, behind one grid barrier; every step
  // after publishes both copies
  if (owner) a.vds[a.step0 & 1][cell] = v.Vd * kVScale;
  bar_target += gridDim.x;
  if (!grid_sync(a, bar_target, &s_abort, nullptr)) return;
  TraceClock tclock(a.trace_every, a.step0);
  for (int st = 0; st < a.n_steps; ++st) {
    const int step = a.step0 + st;
    const bool trace_now = tclock.take();
    const float* vcur = a.vds[step & 1];
    if (owner) sVd[t] = v.Vd * kVScale;
    if (w.n_tiles > 0 && tid == 0) {
      fence_proxy_async_global();
      fence_proxy_async_smem();
      issue_tile(a, vcur, tiles[0], tbuf + (nload % nbuf) * tile_cap, &mbar[nload % nbuf]);
    }
    __syncthreads();
    const float vc = own ? sVd[t] : 0.0f;
    float acc = 0.0f, cmp = 0.0f;
    for (int j = 0; j < w.n_tiles; ++j) {
      const TileDesc td = tiles[j];
      const unsigned k = nload + j;
      const int b = (int)(k % (unsigned)nbuf);
      if (tid == 0 && j > 0 && nbuf == 1) {
        fence_proxy_async_smem();
        issue_tile(a, vcur, td, tbuf, &mbar[0]);
      }
      if (tid == 0 && j + 1 < w.n_tiles && nbuf == 2) {
        fence_proxy_async_smem();
        const int b1 = (int)((k + 1) & 1u);
        issue_tile(a, vcur, tiles[j + 1], tbuf + b1 * tile_cap, &mbar[b1]);
      }
      if (!wait_tile(a, &mbar[b], (k / (unsigned)nbuf) & 1u)) s_abort = 1;
      if (walker) {
        const int c0 = td.chunk_begin, cols = td.chunk_end - td.chunk_begin;
        const int cs = c0 + (int)((long long)cols * slice / S), ce = c0 + (int)((long long)cols * (slice + 1) / S);
        bits_walk<KAHAN>(own, gw, nc, cs, ce, tsm + (uint32_t)b * (uint32_t)tile_cap * 4u, c0, vc, acc, cmp);
      }
      __syncthreads();  // every thread is done with this buffer before it is refilled
    }
    nload += w.n_tiles;
    if (s_abort) break;
    if (own) {
      part[slice * R + t] = acc;
      partc[slice * R + t] = cmp;
    }
    __syncthreads();
    if (owner) {
      float sum = 0.0f, c2 = 0.0f;
      for (int q = 0; q < S; ++q) {
        if (KAHAN) {
          const float y = part[q * R + t] - (partc[q * R + t] + c2);
          const float t2 = sum + y;
          c2 = (t2 - sum) - y;
          sum = t2;
        } else {
          sum += part[q * R + t];
        }
      }
      const float ic = (sum * kInvVScale) * a.g_uniform;  // the sums are in scaled units
      const int ls = step + my_off;
      float iapp;
      if (a.stim_kind == STIM_PULSE)
        iapp = (ls >= a.stim_start && ls < a.stim_end) ? a.stim_amp : 0.0f;
      else if (a.stim_kind == STIM_CELL)
        iapp = (ls >= my_onset && ls < my_onset + a.stim_dur) ? my_amp : 0.0f;
      else
        iapp = a.stim_table[(size_t)st * np + cell];
      Currents cur;
      run_units(a.P, 0xffu, v, g, cur);
      voltage_step(a.P, vk, v, cur, ic, iapp);
      a.vd[(step + 1) & 1][cell] = v.Vd;
      a.vds[(step + 1) & 1][cell] = v.Vd * kVScale;
      if (trace_now) {
        float* tr = a.trace + (size_t)row * a.trace_nq * np + cell;
        int qi = 0;
        if (a.trace_mask & TRACE_AXON) tr[(qi++) * np] = v.Va;
        if (a.trace_mask & TRACE_SOMA) tr[(qi++) * np] = v.Vs;
        if (a.trace_mask & TRACE_DEND) tr[(qi++) * np] = v.Vd;
      }
    }
    if (trace_now) ++row;
    if (st + 1 < a.n_steps) {
      bar_target += gridDim.x;
      if (!grid_sync(a, bar_target, &s_abort, nullptr)) break;
    }
  }
  if (owner) {
    float* stp = a.st;
    stp[F_VS * np + cell] = v.Vs;
    stp[F_VA * np + cell] = v.Va;
    stp[F_Q * np + cell] = g.q;
    stp[F_R * np + cell] = g.r;
    stp[F_S * np + cell] = g.s;
    a.ca[cell] = g.Ca;
    stp[F_ICAH * np + cell] = g.ICaH;
    stp[F_GCAL * np + cell] = g.gCaL;
    stp[F_K * np + cell] = g.k;
    stp[F_L * np + cell] = g.l;
    stp[F_M * np + cell] = g.m;
    stp[F_H * np + cell] = g.h;
    stp[F_N * np + cell] = g.n;
    stp[F_P * np + cell] = g.p;
    stp[F_XS * np + cell] = g.xs;
    stp[F_MA * np + cell] = g.ma;
    stp[F_HA * np + cell] = g.ha;
    stp[F_XA * np + cell] = g.xa;
  }
}

template <int BLOCK, bool K>
cudaError_t launch_bits(const StepArgs& a, int grid, cudaStream_t stream) {
  const size_t smem = tgather_smem_bytes(a.shape);
  auto fn = bits_kernel<BLOCK, K>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(BLOCK), args, smem, stream);
}

template <int BLOCK, bool K, bool G>
cudaError_t launch_tgather(const StepArgs& a, int grid, cudaStream_t stream) {
  const size_t smem = tgather_smem_bytes(a.shape);
  auto fn = tgather_kernel<BLOCK, K, G>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(BLOCK), args, smem, stream);
}

template <int BLOCK, bool K, bool G>
cudaError_t launch_gather(const StepArgs& a, int grid, cudaStream_t stream) {
  const size_t smem = gather_smem_bytes(BLOCK);
  auto fn = gather_kernel<BLOCK, K, G>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(BLOCK), args, smem, stream);
}

template <int BLOCK>
cudaError_t launch_gather_block(const StepArgs& a, int grid, cudaStream_t stream) {
  const bool g = a.edge_g != nullptr;
  if (a.shape.gather == 3) return a.shape.kahan ? launch_bits<BLOCK, true>(a, grid, stream)
                                                 : launch_bits<BLOCK, false>(a, grid, stream);
  if (a.shape.gather == 2) {
    if (a.shape.kahan) return g ? launch_tgather<BLOCK, true, true>(a, grid, stream)
                                : launch_tgather<BLOCK, true, false>(a, grid, stream);
    return g ? launch_tgather<BLOCK, false, true>(a, grid, stream) : launch_tgather<BLOCK, false, false>(a, grid, stream);
  }
  if (a.shape.kahan) return g ? launch_gather<BLOCK, true, true>(a, grid, stream)
                              : launch_gather<BLOCK, true, false>(a, grid, stream);
  return g ? launch_gather<BLOCK, false, true>(a, grid, stream) : launch_gather<BLOCK, false, false>(a, grid, stream);
}

template <int BLOCK, bool K, bool G, bool LL, int NB = kPollBatch>
cudaError_t launch_variant(const StepArgs& a, int grid, size_t smem, cudaStream_t stream) {
  auto fn = step_kernel<BLOCK, K, G, LL, NB>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(BLOCK), args, smem, stream);
}

template <int BLOCK>
cudaError_t launch_block(const StepArgs& a, int grid, size_t smem, cudaStream_t stream) {
  const bool g = a.edge_g != nullptr;
  if (a.shape.stamped) {
    // the small poll batch when every thread's share of the largest window
    // fits in it (one round of loads)
    if (a.shape.poll_words <= kPollBatchSmall * BLOCK) {
      constexpr int S = kPollBatchSmall;
      if (a.shape.kahan) return g ? launch_variant<BLOCK, true, true, true, S>(a, grid, smem, stream)
                                  : launch_variant<BLOCK, true, false, true, S>(a, grid, smem, stream);
      return g ? launch_variant<BLOCK, false, true, true, S>(a, grid, smem, stream)
               : launch_variant<BLOCK, false, false, true, S>(a, grid, smem, stream);
    }
    if (a.shape.kahan) return g ? launch_variant<BLOCK, true, true, true>(a, grid, smem, stream)
                                : launch_variant<BLOCK, true, false, true>(a, grid, smem, stream);
    return g ? launch_variant<BLOCK, false, true, true>(a, grid, smem, stream)
             : launch_variant<BLOCK, false, false, true>(a, grid, smem, stream);
  }
  if (a.shape.kahan) return g ? launch_variant<BLOCK, true, true, false>(a, grid, smem, stream)
                              : launch_variant<BLOCK, true, false, false>(a, grid, smem, stream);
  return g ? launch_variant<BLOCK, false, true, false>(a, grid, smem, stream)
           : launch_variant<BLOCK, false, false, false>(a, grid, smem, stream);
}

}  // namespace

size_t step_kernel_smem(const StepArgs& a) { return smem_layout(a.shape).total; }

cudaError_t launch_step_kernel(const StepArgs& a, int grid, int threads, cudaStream_t stream) {
  if (threads != a.shape.threads) return cudaErrorInvalidValue;
  if (a.shape.gather) {
    if (threads == 1024) return launch_gather_block<1024>(a, grid, stream);
    if (threads == 512) return launch_gather_block<512>(a, grid, stream);
    return cudaErrorInvalidValue;
  }
  const size_t smem = step_kernel_smem(a);
  if (threads == 1024) return launch_block<1024>(a, grid, smem, stream);
  if (threads == 512) return launch_block<512>(a, grid, smem, stream);
  return cudaErrorInvalidValue;
}

int max_coresident_ctas(int threads, size_t smem, cudaError_t* err) {
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    if (threads == 1024) {
      auto fn = step_kernel<1024, false, false, false, kPollBatch>;
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    } else if (threads == 512) {
      auto fn = step_kernel<512, false, false, false, kPollBatch>;
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    } else {
      e = cudaErrorInvalidValue;
    }
  }
  if (err) *err = e;
  if (e != cudaSuccess) return 0;
  return per_sm * nsm;
}

}  // namespace infoli
