// The batched cluster kernel's per-CTA record and the "lane": the serving
// loop's way of running small networks through that kernel, each on device
// buffers of its own, joining and leaving between launches of a few thousand
// steps.  Internal to libinfoli_gpu.so (infoli_batch.cu, infoli_serve.cu).
#pragma once
#include <cstdint>

namespace infoli {

// One CTA slot of a cluster of the batched kernel.  Every CTA of a cluster
// belongs to the same network, so n_steps, step0 and the pulse are the same
// in all of them.
struct alignas(16) BatchCta {
  int net;           // network, -1: idle slot
  int rank;          // rank of this CTA inside its network (0 .. ncta-1)
  int ncta;          // CTAs of the network
  int rank0;         // cluster rank of the network's first CTA (ranks are contiguous)
  int cbeg, ncell;   // owned cells [cbeg, cbeg + ncell), network-local
  int n;             // cells in the network
  int wpr;           // bitmask words per receiver row, ceil(n / 32)
  float* st;         // state: field f of the network's cell c at st[f * T + cell_base + c]
  double* ca;        // Ca2+ of the network's cell c at ca[cell_base + c] (FP64 between launches)
  const uint32_t* bits;  // word w of receiver r at bits[w * n + r] (two zero words after each row)
  long long T;       // SoA stride of st
  long long cell_base;
  float g;           // conductance of every edge of the network
  int resident;      // rows of the owned receivers kept in shared memory
  int cl_sync;       // the cluster holds a network of several CTAs: cluster barrier per step
  int n_steps;       // steps of this launch; < 0: the launch's count
  int step0;         // index of the first step; < 0: the batch's device step counter
  int pulse_start, pulse_end;
  float pulse_amp;
  int pad0;
};

// One network of a lane launch.
struct LaneNet {
  float* st;             // [INFOLI_NSTATE * n] device SoA (reference order; the Ca2+ row is not used)
  double* ca;            // [n] device Ca2+
  const uint32_t* bits;  // [n * (ceil(n/32) + 2)] device rows, infoli__lane_pack_bits layout
  int n;
  float g;
  int step0, n_steps;
  int pulse_start, pulse_end;
  float pulse_amp;
};

}  // namespace infoli

struct infoli_lane;

// Networks of at most this many cells run in the lane (clusters of up to 8
// CTAs of 1,024 threads).
enum { kLaneMaxCells = 8192 };

// Host: a CSR network (receiver rows) as the batched kernel's bitmask rows,
// word-major (word w of receiver r at out[w * n + r]), most-significant bit
// first, self bits cleared, two zero words after every row:
// n * (ceil(n/32) + 2) words.  Returns 0, or -1 for a sender outside [0, n).
int infoli__lane_pack_bits(int n, const int64_t* row_ptr, const int32_t* col, uint32_t* out);
// CTAs (= SMs, one 1,024-thread CTA per SM) a network of n cells takes.
int infoli__lane_ctas(int n);
int infoli__lane_create(int device, const float* params, int kahan, infoli_lane** out);
// Launches n_steps of every network (each its own n_steps, step0 and pulse)
// asynchronously on the lane's streams; nets must stay valid until the
// launch has finished (infoli__lane_query != 0).  The networks' clusters are
// grouped by size, one kernel per group, the groups running concurrently.
int infoli__lane_launch(infoli_lane* L, const infoli::LaneNet* nets, int count);
// 1 when the last launch has finished, 0 while it runs, < 0 on an error.
int infoli__lane_query(infoli_lane* L);
// The lane's own stream (launches are ordered after work queued on it).
void* infoli__lane_stream(infoli_lane* L);
void infoli__lane_destroy(infoli_lane* L);
