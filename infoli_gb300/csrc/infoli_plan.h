// Work decomposition shared by the host planner (infoli_plan.cpp) and the
// persistent step kernel (infoli_kernels.cu).  Plain-old-data only.
//
// A network (or a batch of independent networks laid side by side) is a set
// of receiver cells with CSR neighbour lists into one global V_dend array.
// The planner cuts it into CTA work items:
//   * a CTA owns a contiguous run of cells (<= its thread count); one thread
//     per owned cell runs the fused compartment update, state in registers;
//   * the senders its receivers read form one or more "tiles": contiguous,
//     16-byte-aligned ranges of the V_dend array that are staged into shared
//     memory by a bulk async copy each step;
//   * the edges of a (receiver, tile) pair are cut into chunks of at most
//     kChunkEdges edges (a multiple of it for dense networks, whose slots
//     would not fit in shared memory otherwise); one warp reduces one chunk
//     into one partial-sum slot; the update thread adds its receiver's slots
//     in sender order.
// Edge entries are 16-bit offsets from the tile start (a tile is at most
// 65536 floats), so one gather from shared memory per edge.
//
// Two ways of exchanging V_dend between steps:
//   * barrier mode: V_dend double buffer in global memory, one grid barrier
//     per step, tiles staged by bulk async copies (any window size);
//   * stamped mode (every CTA's window fits in shared memory at once): every
//     cell publishes (V_dend, step) as one 64-bit word into a two-slot array;
//     a CTA polls exactly the words it reads -- its window, the sorted list of
//     its receivers' unique senders, kept in the plan's gcol table at
//     CtaWork::tile_begin (n_tiles entries; stamped plans have no tiles) --
//     plus one word of every CTA that reads it without being read by it, so
//     no slot is overwritten before its readers are done, until their stamps
//     show the step it needs.  No grid barrier: each CTA waits only for its
//     own neighbourhood.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
namespace infoli {
#endif

enum { kChunkEdges = 128, kMaxChunkEdges = 8192 };

// Packed layout of stamped plans.  A lane-chunk is up to kLaneEdges edges of
// one receiver reduced by ONE lane; 32 lane-chunks form a group handled by
// one warp.  Entries are stored transposed in 4-entry quads so lane l reads
// its next four entries with one 8-byte load:
//   entry k of lane l in group g at ((g * kQuads + k / 4) * 32 + l) * 4 + k % 4
// Each entry is the byte offset, from the start of dynamic shared memory, of
// the sender's V_dend; padding entries address the receiver's own V_dend.
enum { kLaneEdges = 32, kQuads = kLaneEdges / 4, kGroupEntries = 32 * kLaneEdges };

typedef struct {
  int cell_begin;   // first owned cell (index into the V_dend / state arrays)
  int n_cells;      // owned cells, <= threads per CTA
  int tile_begin;   // first tile of this CTA in the tile table
  int n_tiles;      // tiles this CTA stages each step
  int slot_begin;   // partial slots of this CTA: chunk ids slot_begin.. (absolute)
  int n_slots;      // number of chunks == number of partial slots
  int probe_begin;  // stamped-exchange mode: cells of CTAs that read this CTA's
  int n_probes;     //   cells but are not read by it (progress probes)
  int group_begin;  // stamped mode: first lane-chunk group of this CTA (absolute)
  int n_groups;     //   number of groups
  int pad0, pad1;
} CtaWork;

typedef struct {
  int lo;           // first V_dend index of the tile (multiple of 4)
  int nfloats;      // tile length in floats (multiple of 4)
  int chunk_begin;  // chunks of this tile: [chunk_begin, chunk_end), absolute
  int chunk_end;
} TileDesc;

typedef struct {
  int slot;         // partial slot, relative to the CTA's slot_begin (first: the
  int recv;         //   kernel loads {slot, recv} as one 8-byte word)
                    // receiver, relative to the CTA's cell_begin
  int edge_begin;   // absolute index into the edge-offset (and per-edge g) arrays
  int count;        // edges in this chunk, 1 .. the plan's chunk length
} ChunkDesc;

#if defined(__CUDACC__)
#define INFOLI_HD __host__ __device__
#else
#define INFOLI_HD
#endif

// Sizes that fix the step kernel's dynamic shared memory.  When res_chunks
// is non-zero the CTA's static work (tile and chunk descriptors, edge
// offsets, per-edge conductances) is copied into shared memory once per
// launch ("resident" plan) instead of being re-read from global memory
// every step.
typedef struct {
  int tile_cap;    // floats per tile buffer
  int nbuf;        // tile buffers (1 or 2)
  int threads;     // threads per CTA
  int cells_cap;   // owned cells per CTA (max over CTAs, multiple of 32)
  int max_slots;   // partial-sum slots per CTA
  int kahan;       // compensated sums (second slot array)
  int res_tiles;   // resident tile descriptors per CTA (0: not resident); stamped
                   // plans keep the window's sender ids there, four per slot
  int res_chunks;  // resident chunk descriptors per CTA (stamped: lane-chunks, 16 B each)
  int res_edges;   // resident edge offsets per CTA
  int edge_g;      // per-edge conductances present
  int stamped;     // stamped exchange (the whole window resident at once, nbuf = 1)
  int dup_words;   // stamped: second copy of the window starts this many floats in
                   // (a multiple of 32 plus 16, so each word sits in two banks 16
                   // apart); 0 = single copy
  int gather;      // 1: gather plan, one thread per receiver reads its senders' V_dend
                   // through L2; edges column by column per CTA (CtaWork::slot_begin
                   // = first entry, pad0 = padded row length); no dynamic shared memory.
                   // 2: tiled gather plan, V_dend staged tile by tile in shared memory
                   // (nbuf x tile_cap floats, then 2 mbarriers), one thread per
                   // receiver; per tile, entries column by column (16-bit offsets from
                   // the tile start; TileDesc::chunk_begin = first entry, chunk_end =
                   // padded row length) and per-receiver counts at CtaWork::slot_begin
                   // + tile * n_cells + receiver.
                   // 3: bitmask plan (uniform g), V_dend staged tile by tile as above;
                   // receivers' adjacency rows as bits (bit 31 of word w = sender 32 w),
                   // word w of local receiver t at CtaWork::slot_begin + w * n_cells + t,
                   // two zero words after each row (CtaWork::pad0 = words per row);
                   // tiles cover whole 32-sender columns (TileDesc::chunk_begin /
                   // chunk_end = first / end column); `slices` threads share a row
  int slices;      // bitmask plan: threads per receiver (column slices)
  int poll_words;  // stamped: the most words one CTA polls per step (window
                   // senders + progress probes); picks the poll batch size
} SmemShape;

static inline INFOLI_HD size_t tgather_smem_bytes(SmemShape s) {
  const size_t tiles = (((size_t)s.nbuf * (size_t)s.tile_cap * sizeof(float) + 15) & ~(size_t)15);
  // bitmask plans: per-slice partial sums (and compensations) of the receivers
  const size_t part =
      s.gather == 3 ? ((size_t)s.slices * 2 + 1) * (size_t)s.cells_cap * sizeof(float) : 0;  // + V_dend
  return tiles + part + 2 * sizeof(uint64_t);
}

// Number of per-cell float arrays kept in shared memory: V_dend, V_soma,
// V_axon and the nine gate-unit currents.
enum { kCellArrays = 13 };
// Stamped plans: cell array 12 holds V_dend x kVScale of the CTA's own cells
// (the window copy holds scaled values too; padding entries read it).
enum { kScaledVArray = 12 };
// Per-cell gate state in shared memory: 17 float fields (indexed like the
// device state arrays) plus the FP64 Ca2+ concentration.
enum { kGateFloats = 17 };

// Dynamic shared-memory layout of the step kernel (byte offsets):
//   [tile buffers: nbuf x tile_cap floats]
//   [cell arrays: kCellArrays x cells_cap floats]
//   [gate state: cells_cap doubles (Ca2+), kGateFloats x cells_cap floats]
//   [partial sums: max_slots floats][Kahan compensations: max_slots floats,
//    16-byte aligned]
//   [2 mbarriers, 16-byte aligned]
//   resident plans only: [tile descs][chunk descs][per-edge g][edge offsets]
typedef struct {
  size_t tiles, vown, gates, gca, part, partc, mbar, tdesc, chunks, eg, edges, total;
} SmemLayout;

static inline INFOLI_HD SmemLayout smem_layout(SmemShape s) {
  SmemLayout L;
  size_t off = 0;
  L.tiles = off;
  off += (size_t)s.nbuf * (size_t)s.tile_cap * sizeof(float);
  L.vown = off;
  off += (size_t)kCellArrays * (size_t)s.cells_cap * sizeof(float);
  off = (off + 7) & ~(size_t)7;
  L.gca = off;
  off += (size_t)s.cells_cap * sizeof(double);
  L.gates = off;
  off += (size_t)kGateFloats * (size_t)s.cells_cap * sizeof(float);
  off = (off + 15) & ~(size_t)15;  // stamped plans read partial slots as float4
  L.part = off;
  off += (size_t)s.max_slots * sizeof(float);
  off = (off + 15) & ~(size_t)15;  // stamped Kahan plans read compensations as float4
  L.partc = off;
  if (s.kahan) off += (size_t)s.max_slots * sizeof(float);
  off = (off + 15) & ~(size_t)15;
  L.mbar = off;
  off += 2 * sizeof(uint64_t);
  L.tdesc = off;
  off += (size_t)s.res_tiles * sizeof(TileDesc);
  L.chunks = off;
  off += (size_t)s.res_chunks * sizeof(ChunkDesc);
  L.eg = off;
  if (s.edge_g) off += (size_t)s.res_edges * sizeof(float);
  L.edges = off;
  off += (size_t)s.res_edges * sizeof(uint16_t);
  off = (off + 15) & ~(size_t)15;
  L.total = off;
  return L;
}

#ifdef __cplusplus
}  // namespace infoli
#endif
