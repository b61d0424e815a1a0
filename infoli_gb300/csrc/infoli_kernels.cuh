// Device-side argument block and launch entry of the persistent step kernel.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "infoli_cell.cuh"
#include "infoli_plan.h"

namespace infoli {

// Per-cell float state arrays on the device (SoA, each n_pad long).  V_dend is
// not here: it lives in the double-buffered vd[2] arrays; Ca2Plus lives in the
// FP64 array `ca`.
enum DevField {
  F_VS = 0, F_VA, F_Q, F_R, F_S, F_ICAH, F_GCAL, F_K, F_L, F_M, F_H, F_N, F_P, F_XS,
  F_MA, F_HA, F_XA, F_COUNT
};

enum StimKind { STIM_PULSE = 0, STIM_CELL = 1, STIM_TABLE = 2 };

enum TraceBits { TRACE_AXON = 1, TRACE_SOMA = 2, TRACE_DEND = 4 };

// Error codes written by the device into *err (0 = fine).
enum DevError {
  DEV_OK = 0,
  DEV_ERR_BARRIER_TIMEOUT = 1,
  DEV_ERR_COPY_TIMEOUT = 2,
  DEV_ERR_CONFIG = 3,
  DEV_ERR_STAMP_TIMEOUT = 4
};

struct StepArgs {
  ModelParams P;
  // work plan
  const CtaWork* cta;
  const TileDesc* tiles;
  const ChunkDesc* chunks;
  const int2* cell_slots;     // per cell {slot_begin relative to CTA, slot_count}
  const uint16_t* edges;      // tile-relative sender offsets
  const float* edge_g;        // per-edge conductance (same order) or nullptr
  const int* gcol;            // gather plans: sender ids, column by column per CTA
  const int* perm;            // relabelled stamped plans: caller's cell id of plan cell i
                              // (state, inputs and traces are in the caller's order); null = same
  const float* cell_g;        // per-cell conductance scale (uniform per network) or nullptr
  float g_uniform;            // used when edge_g and cell_g are both null
  // state
  float* vd[2];               // V_dend double buffer, V^step in vd[step & 1]
  unsigned long long* vll[2]; // stamped mode: (step << 32 | V_dend bits) per cell, slot step & 1
  float* vds[2];              // bitmask plans: V_dend x kVScale (the staged tiles), V^step in vds[step & 1]
  const int* probes;          // stamped mode: progress-probe cells (CtaWork::probe_begin..)
  const int2* gdesc;          // stamped mode: {slot, recv} per lane-chunk (32 per group)
  int n_cells;                // cells in the network (stamped words >= n_cells are never written)
  float* st;                  // F_COUNT x n_pad floats
  double* ca;                 // Ca2Plus, n_pad doubles
  long long n_pad;
  // stimulus
  int stim_kind;
  int stim_start, stim_end;   // STIM_PULSE: amp for start <= step < end
  float stim_amp;
  const float* cell_amp;      // STIM_CELL: per-cell amplitude
  const int* cell_onset;      //            per-cell onset step
  int stim_dur;               //            pulse length in steps
  const float* stim_table;    // STIM_TABLE: [n_steps][n_pad] for this launch
  const int* cell_step_off;   // per-cell offset added to the step index (batched/served), or null
  // steps
  int step0, n_steps;
  // trace
  float* trace;               // [rows][nq][n_pad]
  int trace_every, trace_mask, trace_nq;
  // synchronisation
  unsigned* bar;              // grid barrier counter (zeroed before launch)
  int* err;                   // device error word
  unsigned long long timeout_ns;
  int stall_cta;              // failure-detection test hook: this CTA never arrives at grid
                              // barriers and never publishes stamped words (-1: none), so
                              // the other CTAs' bounded waits run out and report an error
  // shared-memory layout (threads = launch block size)
  SmemShape shape;
  // optional per-CTA phase timers (ns, accumulated): [grid][kProfSlots]
  unsigned long long* prof;
};

// Phase timer slots written when StepArgs::prof is set, in SM cycles: staging
// wait (after the gate units), coupling, update (incl. CTA stragglers), grid
// barrier, steps counted, gate units; and the launch's span in global-timer ns
// and in SM cycles, which converts the others to time.
enum {
  PROF_STAGE = 0, PROF_COUPLE, PROF_UPDATE, PROF_BARRIER, PROF_STEPS, PROF_UNITS, PROF_SPAN_NS,
  PROF_SPAN_CYCLES, kProfSlots = 8
};

// Dynamic shared memory needed for a launch.
size_t step_kernel_smem(const StepArgs& a);

// Cooperative launch of the persistent kernel over `grid` CTAs.
cudaError_t launch_step_kernel(const StepArgs& a, int grid, int threads, cudaStream_t stream);

// Largest co-resident grid for `threads` threads and the given dynamic smem.
int max_coresident_ctas(int threads, size_t smem, cudaError_t* err = nullptr);

}  // namespace infoli
