// Host planner: cuts a CSR network into the CTA / tile / chunk work items of
// the persistent step kernel (see infoli_plan.h for the device-side view).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "infoli_plan.h"

namespace infoli {

// Length of every per-cell device array for n cells: a multiple of 32 with
// 32 spare entries, so tile ends rounded up to 16 bytes stay in bounds.
inline int pad_cells(int n) { return ((n + 31) / 32) * 32 + 32; }

struct alignas(8) int2_t {
  int x, y;
};

struct alignas(8) CellSlots {
  int begin;  // first partial slot, relative to the CTA
  int count;  // number of slots (chunks) of this receiver
};

struct PlanInput {
  int n = 0;                       // receivers 0..n-1 (also the sender id space)
  const int64_t* row_ptr = nullptr;
  const int32_t* col = nullptr;
  const float* g = nullptr;        // per-edge conductance or null
  int grid = 0;                    // CTAs to use (0: heuristic, capped by grid_max)
  int grid_max = 0;                // co-resident CTA limit
  int threads = 1024;              // threads per CTA
  size_t smem_budget = 0;          // dynamic shared memory per CTA (bytes)
  int kahan = 0;
  int no_resident = 0;             // force per-step reads of the static work from global memory
  int sync_mode = 0;               // kSyncAuto / kSyncBarrier / kSyncStamped
  int reorder = 1;                 // stamped plans: try a locality-preserving cell order
  const int* cta_starts = nullptr; // optional CTA cell ranges (grid + 1 entries; internal)
};

// Locality reordering is tried for stamped plans whose largest window is at
// least kReorderMinWindowRatio x the cells per CTA and at most half the
// network, on networks of at most kReorderMaxEdges edges; it is kept when it
// shrinks the largest window by at least a fifth.
enum { kReorderMinWindowRatio = 4, kReorderIters = 160 };
constexpr int64_t kReorderMaxEdges = 32ll << 20;

enum { kSyncAuto = 0, kSyncBarrier = 1, kSyncStamped = 2, kSyncGather = 3, kSyncTiledGather = 4, kSyncBits = 5 };

// Auto mode picks a bitmask plan (uniform g only) over tile/gather plans when
// the density is at least 1 / kBitsMinDensityInv.
enum { kBitsMinDensityInv = 16 };

// Auto mode picks a tiled gather plan over a barrier plan when the mean degree
// is at most this (rows too short to fill a warp per chunk once split by tiles).
enum { kGatherMaxMeanDegree = 384 };

struct Plan {
  int grid = 0, threads = 0, tile_cap = 0, nbuf = 1, max_slots = 0;
  SmemShape shape{};                  // shared-memory shape of the launch
  size_t smem_bytes = 0;
  std::vector<CtaWork> cta;
  std::vector<TileDesc> tiles;
  std::vector<ChunkDesc> chunks;
  std::vector<CellSlots> cell_slots;  // [n]
  std::vector<uint16_t> edges;
  std::vector<float> edge_g;          // empty unless per-edge g
  std::vector<int> probes;            // stamped mode: progress-probe cells
  std::vector<int2_t> gdesc;          // stamped mode: {slot, recv} per lane-chunk, 32 per group
  std::vector<int32_t> gcol;          // gather mode: sender ids, column by column per CTA;
                                      // tiled gather: entries per (tile, receiver);
                                      // bitmask plans: the rows' bit words
  std::vector<int32_t> perm;          // relabelled plans: perm[plan cell] = caller's cell
                                      // (empty: the caller's order); every table above
                                      // uses plan cell ids
};

// Shared-memory bytes the step kernel needs for a plan's parameters.
size_t plan_smem_bytes(int tile_cap, int nbuf, int threads, int cells_cap, int max_slots, int kahan);

// Returns false and sets *err on failure.
bool make_plan(const PlanInput& in, Plan* out, std::string* err);

// Locality-preserving cell order for `parts` CTAs of at most `threads`
// cells: order[new] = old and the CTA starts in the new order (parts + 1
// entries).  Empty when no such order was found.
std::vector<int> locality_order(const PlanInput& in, int parts, int threads, std::vector<int>* starts);

}  // namespace infoli
