// Host planner for the persistent step kernel.  See infoli_plan.h.
#include "infoli_planner.h"

#include <algorithm>
#include <cstdio>
#include <numeric>

namespace infoli {

size_t plan_smem_bytes(int tile_cap, int nbuf, int threads, int max_slots, int kahan) {
  SmemShape s{};
  s.tile_cap = tile_cap;
  s.nbuf = nbuf;
  s.threads = threads;
  s.max_slots = max_slots;
  s.kahan = kahan;
  return smem_layout(s).total;
}

namespace {

constexpr int kCellCost = 8;  // edge-equivalents charged per cell when balancing CTAs

// Contiguous partition of cells into at most `grid` CTAs, each at most
// `threads` cells, minimising the largest per-CTA cost (binary search on the
// bottleneck, greedy packing).  Returns CTA start indices (size = ctas + 1).
std::vector<int> partition_cells(int n, const int64_t* row_ptr, int grid, int threads) {
  auto cost = [&](int c) { return (int64_t)(row_ptr[c + 1] - row_ptr[c]) + kCellCost; };
  int64_t total = 0, maxc = 0;
  for (int c = 0; c < n; ++c) {
    total += cost(c);
    maxc = std::max(maxc, cost(c));
  }
  auto pack = [&](int64_t B, std::vector<int>* starts) {
    int ctas = 0;
    int c = 0;
    if (starts) starts->clear();
    while (c < n) {
      if (starts) starts->push_back(c);
      ++ctas;
      int64_t acc = 0;
      int cnt = 0;
      while (c < n && cnt < threads && acc + cost(c) <= B) {
        acc += cost(c);
        ++cnt;
        ++c;
      }
      if (cnt == 0) {  // single cell above B: cannot happen when B >= maxc
        ++c;
      }
    }
    if (starts) starts->push_back(n);
    return ctas;
  };
  int64_t lo = std::max<int64_t>(maxc, (total + grid - 1) / grid), hi = total;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (pack(mid, nullptr) <= grid)
      hi = mid;
    else
      lo = mid + 1;
  }
  std::vector<int> starts;
  pack(lo, &starts);
  return starts;
}

struct TileSpan {
  int lo, hi;  // [lo, hi) floats, multiples of 4
};

// Tiles covering the sorted unique sender list `u`, each at most `cap` floats.
std::vector<TileSpan> make_tiles(const std::vector<int>& u, int cap, int n_pad) {
  std::vector<TileSpan> t;
  size_t i = 0;
  while (i < u.size()) {
    int lo = u[i] & ~3;
    size_t j = i;
    while (j + 1 < u.size() && u[j + 1] < lo + cap) ++j;
    int hi = std::min(n_pad, (u[j] + 1 + 3) & ~3);
    t.push_back({lo, hi});
    i = j + 1;
  }
  return t;
}

}  // namespace

bool make_plan(const PlanInput& in, Plan* out, std::string* err) {
  const int n = in.n;
  if (n <= 0 || !in.row_ptr || in.threads <= 0 || in.threads % 32 || in.grid_max <= 0) {
    *err = "make_plan: bad input";
    return false;
  }
  const int64_t E = in.row_ptr[n];
  if (E > 0 && !in.col) {
    *err = "make_plan: missing col";
    return false;
  }
  for (int c = 0; c < n; ++c)
    if (in.row_ptr[c + 1] < in.row_ptr[c]) {
      *err = "make_plan: row_ptr not monotone";
      return false;
    }
  for (int64_t e = 0; e < E; ++e)
    if (in.col[e] < 0 || in.col[e] >= n) {
      char b[128];
      snprintf(b, sizeof b, "make_plan: sender id %d out of range at edge %lld", in.col[e], (long long)e);
      *err = b;
      return false;
    }
  if (E > INT32_MAX) {
    *err = "make_plan: more than 2^31-1 edges";
    return false;
  }
  const int threads = in.threads;
  const int nwarps = threads / 32;
  const int n_pad = pad_cells(n);

  // ---- grid size: enough CTAs that every warp gets about two chunks
  int grid = in.grid;
  if (grid <= 0) {
    const int64_t per_cta = (int64_t)nwarps * kChunkEdges * 2;
    grid = (int)std::min<int64_t>(in.grid_max, std::max<int64_t>(1, (E + per_cta - 1) / per_cta));
    grid = std::max(grid, (n + threads - 1) / threads);
  }
  grid = std::min(grid, in.grid_max);
  if ((int64_t)grid * threads < n) {
    *err = "make_plan: network larger than the co-resident thread count";
    return false;
  }
  std::vector<int> starts = partition_cells(n, in.row_ptr, grid, threads);
  const int ctas = (int)starts.size() - 1;

  // ---- per-CTA sorted edges (sender, g) and unique sender lists
  std::vector<std::vector<int>> uniq(ctas);
  int max_window = 4;
  for (int b = 0; b < ctas; ++b) {
    std::vector<int>& u = uniq[b];
    for (int c = starts[b]; c < starts[b + 1]; ++c)
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) u.push_back(in.col[e]);
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    if (!u.empty()) max_window = std::max(max_window, ((u.back() + 4) & ~3) - (u.front() & ~3));
  }

  // ---- tile capacity: one buffer holding the whole window when it fits,
  // otherwise two buffers for overlapped staging; shrink until smem fits.
  auto slots_for = [&](int b, const std::vector<TileSpan>& tl) {
    int s = 0;
    for (int c = starts[b]; c < starts[b + 1]; ++c) {
      // edges of c split by tile, then by chunk size
      int64_t e = in.row_ptr[c], e1 = in.row_ptr[c + 1];
      std::vector<int> snd(in.col + e, in.col + e1);
      std::sort(snd.begin(), snd.end());
      size_t k = 0;
      for (const TileSpan& t : tl) {
        int cnt = 0;
        while (k < snd.size() && snd[k] < t.hi) {
          ++cnt;
          ++k;
        }
        s += (cnt + kChunkEdges - 1) / kChunkEdges;
      }
    }
    return s;
  };
  int nbuf = 1, tile_cap = std::min(max_window, 65536);
  std::vector<std::vector<TileSpan>> tiles(ctas);
  int max_slots = 0;
  for (int attempt = 0; attempt < 16; ++attempt) {
    if (max_window > tile_cap) nbuf = 2;
    max_slots = 0;
    for (int b = 0; b < ctas; ++b) {
      tiles[b] = make_tiles(uniq[b], tile_cap, n_pad);
      max_slots = std::max(max_slots, slots_for(b, tiles[b]));
    }
    max_slots = std::max(max_slots, 1);
    if (plan_smem_bytes(tile_cap, nbuf, threads, max_slots, in.kahan) <= in.smem_budget) break;
    // shrink: give the tiles what is left after the fixed part
    size_t fixed = plan_smem_bytes(0, 0, threads, max_slots, in.kahan);
    size_t avail = in.smem_budget > fixed ? in.smem_budget - fixed : 0;
    int cap = (int)std::min<size_t>(avail / (2 * sizeof(float)), (size_t)tile_cap * 3 / 4);
    cap &= ~3;
    if (cap < 256) {
      *err = "make_plan: shared memory budget too small";
      return false;
    }
    tile_cap = cap;
    nbuf = 2;
  }
  if (plan_smem_bytes(tile_cap, nbuf, threads, max_slots, in.kahan) > in.smem_budget) {
    *err = "make_plan: could not fit shared memory";
    return false;
  }

  // ---- build CTA / tile / chunk tables
  Plan& P = *out;
  P = Plan();
  P.grid = ctas;
  P.threads = threads;
  P.tile_cap = tile_cap;
  P.nbuf = nbuf;
  P.max_slots = max_slots;
  P.smem_bytes = plan_smem_bytes(tile_cap, nbuf, threads, max_slots, in.kahan);
  P.cell_slots.assign(n, CellSlots{0, 0});
  P.edges.reserve(E);
  if (in.g) P.edge_g.reserve(E);
  int slot_base = 0;
  struct PendingChunk {
    int tile, recv, slot;
    std::vector<std::pair<int, float>> e;  // (sender, g)
  };
  for (int b = 0; b < ctas; ++b) {
    CtaWork w{};
    w.cell_begin = starts[b];
    w.n_cells = starts[b + 1] - starts[b];
    w.tile_begin = (int)P.tiles.size();
    w.n_tiles = (int)tiles[b].size();
    w.slot_begin = slot_base;
    const std::vector<TileSpan>& tl = tiles[b];
    std::vector<PendingChunk> pend;
    int slot = 0;
    for (int r = 0; r < w.n_cells; ++r) {
      const int c = w.cell_begin + r;
      std::vector<std::pair<int, float>> snd;
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e)
        snd.push_back({in.col[e], in.g ? in.g[e] : 0.0f});
      std::stable_sort(snd.begin(), snd.end(),
                       [](const std::pair<int, float>& x, const std::pair<int, float>& y) { return x.first < y.first; });
      P.cell_slots[c].begin = slot;
      size_t k = 0;
      for (int j = 0; j < (int)tl.size(); ++j) {
        std::vector<std::pair<int, float>> in_tile;
        while (k < snd.size() && snd[k].first < tl[j].hi) in_tile.push_back(snd[k++]);
        for (size_t o = 0; o < in_tile.size(); o += kChunkEdges) {
          PendingChunk pc;
          pc.tile = j;
          pc.recv = r;
          pc.slot = slot++;
          pc.e.assign(in_tile.begin() + o, in_tile.begin() + std::min(in_tile.size(), o + kChunkEdges));
          pend.push_back(std::move(pc));
        }
      }
      P.cell_slots[c].count = slot - P.cell_slots[c].begin;
    }
    w.n_slots = slot;
    // tile-major; inside a tile, larger chunks first (round-robin to warps)
    std::stable_sort(pend.begin(), pend.end(), [](const PendingChunk& x, const PendingChunk& y) {
      if (x.tile != y.tile) return x.tile < y.tile;
      return x.e.size() > y.e.size();
    });
    size_t pi = 0;
    for (int j = 0; j < (int)tl.size(); ++j) {
      TileDesc td{};
      td.lo = tl[j].lo;
      td.nfloats = tl[j].hi - tl[j].lo;
      td.chunk_begin = (int)P.chunks.size();
      while (pi < pend.size() && pend[pi].tile == j) {
        const PendingChunk& pc = pend[pi++];
        ChunkDesc cd{};
        cd.edge_begin = (int)P.edges.size();
        cd.slot = pc.slot;
        cd.recv = pc.recv;
        cd.count = (int)pc.e.size();
        for (const auto& se : pc.e) {
          P.edges.push_back((uint16_t)(se.first - td.lo));
          if (in.g) P.edge_g.push_back(se.second);
        }
        P.chunks.push_back(cd);
      }
      td.chunk_end = (int)P.chunks.size();
      P.tiles.push_back(td);
    }
    slot_base += slot;
    P.cta.push_back(w);
  }

  // ---- shared-memory shape; keep the static work resident when it fits
  SmemShape sh{};
  sh.tile_cap = tile_cap;
  sh.nbuf = nbuf;
  sh.threads = threads;
  sh.max_slots = max_slots;
  sh.kahan = in.kahan;
  sh.edge_g = in.g ? 1 : 0;
  int mt = 0, mc = 0, me = 0;
  for (const CtaWork& w : P.cta) {
    if (w.n_tiles == 0) continue;
    const int c0 = P.tiles[w.tile_begin].chunk_begin, c1 = P.tiles[w.tile_begin + w.n_tiles - 1].chunk_end;
    const int e0 = c1 > c0 ? P.chunks[c0].edge_begin : 0;
    const int e1 = c1 > c0 ? P.chunks[c1 - 1].edge_begin + P.chunks[c1 - 1].count : 0;
    mt = std::max(mt, w.n_tiles);
    mc = std::max(mc, c1 - c0);
    me = std::max(me, e1 - e0);
  }
  SmemShape res = sh;
  res.res_tiles = std::max(mt, 1);
  res.res_chunks = std::max(mc, 1);
  res.res_edges = std::max(me, 1);
  if (!in.no_resident && smem_layout(res).total <= in.smem_budget) sh = res;
  P.shape = sh;
  P.smem_bytes = smem_layout(sh).total;
  return true;
}

}  // namespace infoli
