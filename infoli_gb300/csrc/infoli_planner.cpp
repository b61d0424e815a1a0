// Host planner for the persistent step kernel.  See infoli_plan.h.
#include "infoli_planner.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>

namespace infoli {

size_t plan_smem_bytes(int tile_cap, int nbuf, int threads, int cells_cap, int max_slots, int kahan) {
  SmemShape s{};
  s.tile_cap = tile_cap;
  s.nbuf = nbuf;
  s.threads = threads;
  s.cells_cap = cells_cap;
  s.max_slots = max_slots;
  s.kahan = kahan;
  return smem_layout(s).total;
}

namespace {

constexpr int kCellCost = 8;  // edge-equivalents charged per cell when balancing CTAs
constexpr int kSmallNetworkCtas = 100;  // the most CTAs the small-network floor asks for

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

// Build the packed lane-chunk tables of a stamped, resident plan (see
// infoli_plan.h): per receiver, its senders (ascending) become byte offsets
// into the CTA's window (its sorted unique senders, win[b], one float each),
// cut into lane-chunks of kLaneEdges;
// the chunks of a CTA, receiver-major, are dealt 32 per group.  Inside a
// group, entries are permuted per chunk so that the 32 lanes reading
// position k hit distinct shared-memory banks where possible.  Receiver slots
// are rewritten to the lane-chunks (receiver-major, so a receiver's partial
// sums stay contiguous and in sender order); the last group of a CTA is
// filled with dummy chunks that write one spare slot.
void pack_groups(Plan& P, const SmemLayout& L, const PlanInput& in, const std::vector<std::vector<int>>& win,
                 int dup_words, int cells_cap) {
  const bool edge_g = in.g != nullptr;
  // CTAs are packed in parallel into local tables, then concatenated
  struct Local {
    std::vector<int2_t> gdesc;
    std::vector<uint16_t> pe;
    std::vector<float> pg;
  };
  const int ctas = (int)P.cta.size();
  std::vector<Local> loc(ctas);
  int max_slots = 1;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : max_slots)
  for (int b = 0; b < ctas; ++b) {
    CtaWork& w = P.cta[b];
    std::vector<int2_t>& gdesc = loc[b].gdesc;
    std::vector<uint16_t>& pe = loc[b].pe;
    std::vector<float>& pg = loc[b].pg;
    const std::vector<int>& u = win[b];
    struct LaneChunk {
      int recv, slot;
      std::vector<std::pair<uint16_t, float>> e;
    };
    std::vector<LaneChunk> lc;
    int slot = 0, prev_begin = 0;
    for (int r = 0; r < w.n_cells; ++r) {
      const int c = w.cell_begin + r;
      std::vector<std::pair<int, float>> snd;
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) snd.push_back({in.col[e], edge_g ? in.g[e] : 0.0f});
      std::stable_sort(snd.begin(), snd.end(),
                       [](const std::pair<int, float>& x, const std::pair<int, float>& y) { return x.first < y.first; });
      // each receiver's partial slots start on a 4-slot (16-byte) boundary; the
      // gaps are zeroed once per launch, so the update can read them 4 at a time.
      // Consecutive receivers start an odd number of 16-byte units apart (an
      // unread unit is added after an even-sized block), so the 8 lanes of each
      // phase of a 16-byte shared-memory load (one receiver per lane) fall in
      // 8 different bank groups instead of 2
      slot = (slot + 3) & ~3;
      if (r > 0 && (((slot - prev_begin) >> 2) & 1) == 0) slot += 4;
      prev_begin = slot;
      P.cell_slots[c].begin = slot;
      size_t j = 0;  // window position of the sender (senders ascending)
      for (size_t k = 0; k < snd.size(); k += kLaneEdges) {
        LaneChunk ch;
        ch.recv = r;
        ch.slot = slot++;
        for (size_t q = k; q < std::min(snd.size(), k + kLaneEdges); ++q) {
          const int s = snd[q].first;
          while (u[j] < s) ++j;
          ch.e.push_back({(uint16_t)(L.tiles + sizeof(float) * j), snd[q].second});
        }
        lc.push_back(std::move(ch));
      }
      P.cell_slots[c].count = slot - P.cell_slots[c].begin;
    }
    const int dummy_slot = (slot + 3) & ~3;  // past the last receiver's 4-slot block
    w.n_slots = dummy_slot;
    max_slots = std::max(max_slots, dummy_slot + 1);
    const int ng = (int)(lc.size() + 31) / 32;
    w.n_groups = ng;
    for (int g = 0; g < ng; ++g) {
      // the 32 chunks of this group (dummies past the end)
      std::vector<std::vector<std::pair<uint16_t, float>>> rem(32);
      std::vector<uint16_t> pad(32);
      for (int l = 0; l < 32; ++l) {
        const size_t ci = (size_t)g * 32 + l;
        int2_t d;
        if (ci < lc.size()) {
          d.x = lc[ci].slot;
          d.y = lc[ci].recv;
          rem[l] = lc[ci].e;
        } else {
          d.x = dummy_slot;
          d.y = 0;
        }
        pad[l] = (uint16_t)(L.vown + sizeof(float) * ((size_t)kScaledVArray * cells_cap + d.y));
        gdesc.push_back(d);
      }
      // bank-distinct dealing, position by position: lanes whose chunk is
      // exhausted read their padding word (lanes of one receiver share it);
      // the others are matched to free banks by augmenting paths (Kuhn), so
      // each position has as many conflict-free lanes as the remaining
      // entries allow; unmatched lanes take any entry
      std::vector<std::pair<uint16_t, float>> cell(32 * kLaneEdges);
      for (int k = 0; k < kLaneEdges; ++k) {
        int bank_word[32];
        for (int b2 = 0; b2 < 32; ++b2) bank_word[b2] = -1;
        for (int l = 0; l < 32; ++l)
          if (rem[l].empty()) {
            cell[l * kLaneEdges + k] = {pad[l], 0.0f};
            const int wd = pad[l] >> 2;
            if (bank_word[wd & 31] < 0) bank_word[wd & 31] = wd;
          }
        // an entry can be read from the first copy (bank b) or, when the
        // window is duplicated, from the second (bank b + 16)
        const unsigned dup_mask = dup_words ? 0xffffffffu : 0u;
        auto banks_of = [&](uint16_t off) {
          const int b2 = (off >> 2) & 31;
          return (1u << b2) | (dup_mask & (1u << ((b2 + 16) & 31)));
        };
        unsigned taken = 0;  // banks already claimed by padding words
        for (int b2 = 0; b2 < 32; ++b2)
          if (bank_word[b2] >= 0) taken |= 1u << b2;
        unsigned adj[32];
        for (int l = 0; l < 32; ++l) {
          adj[l] = 0;
          for (const auto& e : rem[l]) adj[l] |= banks_of(e.first);
          adj[l] &= ~taken;
        }
        int match_bank[32];  // bank -> lane
        for (int b2 = 0; b2 < 32; ++b2) match_bank[b2] = -1;
        for (int l = 0; l < 32; ++l) {
          if (!adj[l]) continue;
          unsigned seen = 0;
          // iterative augmenting-path search from lane l
          struct Frame {
            int lane;
            unsigned left;
          };
          Frame stack[33];
          int prev_bank[33];
          int sp = 0;
          stack[0] = {l, adj[l]};
          bool done = false;
          while (sp >= 0 && !done) {
            Frame& f = stack[sp];
            const unsigned cand = f.left & ~seen;
            if (!cand) {
              --sp;
              continue;
            }
            const int b2 = __builtin_ctz(cand);
            f.left &= ~(1u << b2);
            seen |= 1u << b2;
            prev_bank[sp] = b2;
            if (match_bank[b2] < 0) {
              for (int q = sp; q >= 0; --q) match_bank[prev_bank[q]] = stack[q].lane;
              done = true;
            } else if (sp + 1 < 33) {
              ++sp;
              stack[sp] = {match_bank[b2], adj[match_bank[b2]]};
            }
          }
        }
        int lane_bank[32];
        for (int l = 0; l < 32; ++l) lane_bank[l] = -1;
        for (int b2 = 0; b2 < 32; ++b2)
          if (match_bank[b2] >= 0) lane_bank[match_bank[b2]] = b2;
        for (int l = 0; l < 32; ++l) {
          if (rem[l].empty()) continue;
          size_t q = 0;
          std::pair<uint16_t, float> pick = rem[l][0];
          if (lane_bank[l] >= 0) {
            while (!(banks_of(rem[l][q].first) & (1u << lane_bank[l]))) ++q;
            pick = rem[l][q];
            if (((pick.first >> 2) & 31) != lane_bank[l])  // the matched bank is the second copy's
              pick.first = (uint16_t)(pick.first + sizeof(float) * (size_t)dup_words);
          }
          cell[l * kLaneEdges + k] = pick;
          rem[l].erase(rem[l].begin() + q);
        }
      }
      // transposed quads: ((g * kQuads + k / 4) * 32 + l) * 4 + k % 4
      const size_t base = pe.size();
      pe.resize(base + kGroupEntries);
      if (edge_g) pg.resize(base + kGroupEntries);
      for (int l = 0; l < 32; ++l)
        for (int k = 0; k < kLaneEdges; ++k) {
          const size_t at = base + ((size_t)(k / 4) * 32 + l) * 4 + (k % 4);
          pe[at] = cell[l * kLaneEdges + k].first;
          if (edge_g) pg[at] = cell[l * kLaneEdges + k].second;
        }
    }
  }
  std::vector<int2_t> gdesc;
  std::vector<uint16_t> pe;
  std::vector<float> pg;
  for (int b = 0; b < ctas; ++b) {
    P.cta[b].group_begin = (int)(gdesc.size() / 32);
    gdesc.insert(gdesc.end(), loc[b].gdesc.begin(), loc[b].gdesc.end());
    pe.insert(pe.end(), loc[b].pe.begin(), loc[b].pe.end());
    pg.insert(pg.end(), loc[b].pg.begin(), loc[b].pg.end());
    Local().gdesc.swap(loc[b].gdesc);
    Local().pe.swap(loc[b].pe);
    Local().pg.swap(loc[b].pg);
  }
  P.gdesc.swap(gdesc);
  P.edges.swap(pe);
  P.edge_g.swap(pg);
  P.max_slots = max_slots;
}

}  // namespace

// Gather plan: cells partitioned over the CTAs by edge count (plus a per-cell
// cost), each CTA's rows stored column by column and padded to its longest
// row with the receiver itself (V = 0, so a pad adds exactly 0).
static bool make_gather_plan(const PlanInput& in, Plan* out, std::string* err) {
  const int n = in.n, threads = in.threads;
  int grid = in.grid > 0 ? in.grid : in.grid_max;
  grid = std::min(grid, in.grid_max);
  grid = std::max(grid, (n + threads - 1) / threads);
  if (grid > in.grid_max) {
    *err = "make_plan: network larger than the co-resident thread count";
    return false;
  }
  std::vector<int> starts = partition_cells(n, in.row_ptr, grid, threads);
  const int ctas = (int)starts.size() - 1;
  Plan& P = *out;
  P = Plan();
  P.grid = ctas;
  P.threads = threads;
  P.cta.resize(ctas);
  int64_t total = 0;
  int cells_cap = 32;
  for (int b = 0; b < ctas; ++b) {
    int deg = 0;
    for (int c = starts[b]; c < starts[b + 1]; ++c) deg = std::max<int>(deg, (int)(in.row_ptr[c + 1] - in.row_ptr[c]));
    CtaWork& w = P.cta[b];
    w = CtaWork{};
    w.cell_begin = starts[b];
    w.n_cells = starts[b + 1] - starts[b];
    w.slot_begin = (int)std::min<int64_t>(total, INT32_MAX);
    w.pad0 = deg;
    total += (int64_t)deg * w.n_cells;
    cells_cap = std::max(cells_cap, ((w.n_cells + 31) / 32) * 32);
  }
  if (total > INT32_MAX) {
    *err = "make_plan: gather plan needs more than 2^31-1 entries";
    return false;
  }
  P.gcol.assign((size_t)total, 0);
  if (in.g) P.edge_g.assign((size_t)total, 0.0f);
  for (int b = 0; b < ctas; ++b) {
    const CtaWork& w = P.cta[b];
    for (int t = 0; t < w.n_cells; ++t) {
      const int c = w.cell_begin + t;
      const int64_t e0 = in.row_ptr[c], len = in.row_ptr[c + 1] - e0;
      for (int j = 0; j < w.pad0; ++j) {
        const size_t at = (size_t)w.slot_begin + (size_t)j * w.n_cells + t;
        P.gcol[at] = j < len ? in.col[e0 + j] : c;
        if (in.g) P.edge_g[at] = j < len ? in.g[e0 + j] : 0.0f;
      }
    }
  }
  P.cell_slots.assign(n, CellSlots{0, 0});
  P.shape = SmemShape{};
  P.shape.threads = threads;
  P.shape.cells_cap = cells_cap;
  P.shape.kahan = in.kahan;
  P.shape.edge_g = in.g != nullptr;
  P.shape.gather = 1;
  P.smem_bytes = 0;
  return true;
}

// Tiled gather plan: like the gather plan, one thread per receiver, but the
// senders' V_dend are staged tile by tile into shared memory by bulk copies;
// per tile, a receiver's senders in that tile (ascending) are stored column by
// column as 16-bit tile offsets, with per-receiver counts.
static bool make_tgather_plan(const PlanInput& in, Plan* out, std::string* err) {
  const int n = in.n, threads = in.threads;
  const int n_pad = pad_cells(n);
  int grid = in.grid > 0 ? in.grid : in.grid_max;
  grid = std::min(grid, in.grid_max);
  grid = std::max(grid, (n + threads - 1) / threads);
  if (grid > in.grid_max) {
    *err = "make_plan: network larger than the co-resident thread count";
    return false;
  }
  std::vector<int> starts = partition_cells(n, in.row_ptr, grid, threads);
  const int ctas = (int)starts.size() - 1;
  // per-CTA unique senders and window
  std::vector<std::vector<int>> uniq(ctas);
  int max_window = 4;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : max_window)
  for (int b = 0; b < ctas; ++b) {
    std::vector<int>& u = uniq[b];
    for (int c = starts[b]; c < starts[b + 1]; ++c)
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) u.push_back(in.col[e]);
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    if (!u.empty()) max_window = std::max(max_window, ((u.back() + 4) & ~3) - (u.front() & ~3));
  }
  SmemShape sh{};
  sh.threads = threads;
  sh.kahan = in.kahan;
  sh.edge_g = in.g != nullptr;
  sh.gather = 2;
  // one buffer when a CTA's window fits; else two half-size buffers, so the
  // next tile's copy overlaps this tile's gathers
  const size_t avail = in.smem_budget > 64 ? in.smem_budget - 64 : 0;
  const int cap1 = (int)std::min<size_t>(65536, avail / sizeof(float)) & ~3;
  if (cap1 < 256) {
    *err = "make_plan: shared memory budget too small";
    return false;
  }
  if (((max_window + 3) & ~3) <= cap1) {
    sh.nbuf = 1;
    sh.tile_cap = (max_window + 3) & ~3;
  } else {
    sh.nbuf = 2;
    sh.tile_cap = std::min(65536, (int)(avail / (2 * sizeof(float)))) & ~3;
  }
  std::vector<std::vector<TileSpan>> tiles(ctas);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < ctas; ++b) tiles[b] = make_tiles(uniq[b], sh.tile_cap, n_pad);
  // per CTA local tables, then concatenation
  struct Local {
    std::vector<TileDesc> tiles;
    std::vector<uint16_t> edges;
    std::vector<float> edge_g;
    std::vector<int32_t> counts;
  };
  std::vector<Local> loc(ctas);
  int cells_cap = 32;
  for (int b = 0; b < ctas; ++b) cells_cap = std::max(cells_cap, ((starts[b + 1] - starts[b] + 31) / 32) * 32);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < ctas; ++b) {
    Local& L = loc[b];
    const int nc = starts[b + 1] - starts[b];
    const std::vector<TileSpan>& tl = tiles[b];
    // sorted senders per receiver (stable: equal ids keep their order)
    std::vector<std::vector<std::pair<int, float>>> rows(nc);
    for (int t = 0; t < nc; ++t) {
      const int c = starts[b] + t;
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) rows[t].push_back({in.col[e], in.g ? in.g[e] : 0.0f});
      std::stable_sort(rows[t].begin(), rows[t].end(),
                       [](const std::pair<int, float>& x, const std::pair<int, float>& y) { return x.first < y.first; });
    }
    std::vector<size_t> pos(nc, 0);
    L.counts.assign((size_t)tl.size() * nc, 0);
    for (int j = 0; j < (int)tl.size(); ++j) {
      // this tile's range of each row
      std::vector<size_t> end(nc);
      int deg = 0;
      for (int t = 0; t < nc; ++t) {
        size_t k = pos[t];
        while (k < rows[t].size() && rows[t][k].first < tl[j].hi) ++k;
        end[t] = k;
        L.counts[(size_t)j * nc + t] = (int32_t)(k - pos[t]);
        deg = std::max<int>(deg, (int)(k - pos[t]));
      }
      TileDesc td{};
      td.lo = tl[j].lo;
      td.nfloats = tl[j].hi - tl[j].lo;
      td.chunk_begin = (int)L.edges.size();  // local; made absolute below
      td.chunk_end = deg;
      L.edges.resize(L.edges.size() + (size_t)deg * nc, 0);
      if (in.g) L.edge_g.resize(L.edge_g.size() + (size_t)deg * nc, 0.0f);
      for (int t = 0; t < nc; ++t)
        for (size_t k = pos[t]; k < end[t]; ++k) {
          const size_t at = (size_t)td.chunk_begin + (k - pos[t]) * nc + t;
          L.edges[at] = (uint16_t)(rows[t][k].first - td.lo);
          if (in.g) L.edge_g[at] = rows[t][k].second;
        }
      for (int t = 0; t < nc; ++t) pos[t] = end[t];
      L.tiles.push_back(td);
    }
  }
  Plan& P = *out;
  P = Plan();
  P.grid = ctas;
  P.threads = threads;
  P.tile_cap = sh.tile_cap;
  P.nbuf = sh.nbuf;
  P.cell_slots.assign(n, CellSlots{0, 0});
  int64_t total_e = 0, total_c = 0;
  for (int b = 0; b < ctas; ++b) {
    total_e += (int64_t)loc[b].edges.size();
    total_c += (int64_t)loc[b].counts.size();
  }
  if (total_e > INT32_MAX || total_c > INT32_MAX) {
    *err = "make_plan: tiled gather plan needs more than 2^31-1 entries";
    return false;
  }
  P.edges.reserve((size_t)total_e);
  if (in.g) P.edge_g.reserve((size_t)total_e);
  P.gcol.reserve((size_t)total_c);
  for (int b = 0; b < ctas; ++b) {
    Local& L = loc[b];
    CtaWork w{};
    w.cell_begin = starts[b];
    w.n_cells = starts[b + 1] - starts[b];
    w.tile_begin = (int)P.tiles.size();
    w.n_tiles = (int)L.tiles.size();
    w.slot_begin = (int)P.gcol.size();
    const int e0 = (int)P.edges.size();
    for (TileDesc td : L.tiles) {
      td.chunk_begin += e0;
      P.tiles.push_back(td);
    }
    P.edges.insert(P.edges.end(), L.edges.begin(), L.edges.end());
    if (in.g) P.edge_g.insert(P.edge_g.end(), L.edge_g.begin(), L.edge_g.end());
    P.gcol.insert(P.gcol.end(), L.counts.begin(), L.counts.end());
    P.cta.push_back(w);
    Local().edges.swap(L.edges);
  }
  sh.cells_cap = cells_cap;
  sh.res_tiles = 0;
  P.shape = sh;
  P.smem_bytes = tgather_smem_bytes(sh);
  if (P.smem_bytes > in.smem_budget) {
    *err = "make_plan: could not fit shared memory";
    return false;
  }
  return true;
}

// Bitmask plan (uniform conductance): cells partitioned over the CTAs; every
// CTA stages the whole V_dend array tile by tile (tiles of whole 32-sender
// columns) and its receivers walk their adjacency bits column by column in
// warp lockstep, `slices` threads per receiver each taking a share of the
// columns of every tile.
static bool make_bits_plan(const PlanInput& in, Plan* out, std::string* err) {
  const int n = in.n, threads = in.threads;
  if (in.g) {
    *err = "make_plan: bitmask plans need a uniform conductance";
    return false;
  }
  int grid = in.grid > 0 ? in.grid : in.grid_max;
  grid = std::min(grid, in.grid_max);
  grid = std::max(grid, (n + threads - 1) / threads);
  if (grid > in.grid_max) {
    *err = "make_plan: network larger than the co-resident thread count";
    return false;
  }
  std::vector<int> starts = partition_cells(n, in.row_ptr, grid, threads);
  const int ctas = (int)starts.size() - 1;
  int cells_cap = 32;
  for (int b = 0; b < ctas; ++b) cells_cap = std::max(cells_cap, ((starts[b + 1] - starts[b] + 31) / 32) * 32);
  const int wpr = (n + 31) / 32;
  SmemShape sh{};
  sh.threads = threads;
  sh.kahan = in.kahan;
  sh.edge_g = 0;
  sh.gather = 3;
  sh.cells_cap = cells_cap;
  sh.slices = std::max(1, std::min(8, threads / cells_cap));
  const size_t part = ((size_t)sh.slices * 2 + 1) * cells_cap * sizeof(float);
  const size_t avail = in.smem_budget > part + 64 ? in.smem_budget - part - 64 : 0;
  const int window = wpr * 32;
  const int cap1 = (int)std::min<size_t>(65536, avail / sizeof(float)) & ~31;
  if (cap1 < 1024) {
    *err = "make_plan: shared memory budget too small";
    return false;
  }
  if (window <= cap1) {
    sh.nbuf = 1;
    sh.tile_cap = window;
  } else {
    sh.nbuf = 2;
    sh.tile_cap = (int)std::min<size_t>(65536, avail / (2 * sizeof(float))) & ~31;
  }
  Plan& P = *out;
  P = Plan();
  P.grid = ctas;
  P.threads = threads;
  P.tile_cap = sh.tile_cap;
  P.nbuf = sh.nbuf;
  P.cell_slots.assign(n, CellSlots{0, 0});
  int64_t total = 0;
  for (int b = 0; b < ctas; ++b) total += (int64_t)(starts[b + 1] - starts[b]) * (wpr + 2);
  if (total > INT32_MAX) {
    *err = "make_plan: bitmask plan needs more than 2^31-1 words";
    return false;
  }
  P.gcol.assign((size_t)total, 0);
  // tiles: the same column ranges for every CTA
  std::vector<TileDesc> tl;
  const int tcols = sh.tile_cap / 32;
  for (int c0 = 0; c0 < wpr; c0 += tcols) {
    TileDesc td{};
    td.lo = c0 * 32;
    const int c1 = std::min(wpr, c0 + tcols);
    td.nfloats = std::min((c1 - c0) * 32, pad_cells(n) - td.lo);
    td.chunk_begin = c0;
    td.chunk_end = c1;
    tl.push_back(td);
  }
  int64_t base = 0;
  for (int b = 0; b < ctas; ++b) {
    CtaWork w{};
    w.cell_begin = starts[b];
    w.n_cells = starts[b + 1] - starts[b];
    w.tile_begin = (int)P.tiles.size();
    w.n_tiles = (int)tl.size();
    w.slot_begin = (int)base;
    w.pad0 = wpr;
    P.tiles.insert(P.tiles.end(), tl.begin(), tl.end());
    P.cta.push_back(w);
    base += (int64_t)w.n_cells * (wpr + 2);
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < ctas; ++b) {
    const CtaWork& w = P.cta[b];
    uint32_t* bits = reinterpret_cast<uint32_t*>(P.gcol.data()) + w.slot_begin;
    for (int t = 0; t < w.n_cells; ++t) {
      const int c = w.cell_begin + t;
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) {
        const int s = in.col[e];
        if (s == c) continue;  // no self-coupling (adds 0 anyway)
        bits[(size_t)(s >> 5) * w.n_cells + t] |= 0x80000000u >> (s & 31);
      }
    }
  }
  P.shape = sh;
  P.smem_bytes = tgather_smem_bytes(sh);
  if (P.smem_bytes > in.smem_budget) {
    *err = "make_plan: could not fit shared memory";
    return false;
  }
  return true;
}

bool make_plan_base(const PlanInput& in, Plan* out, std::string* err) {
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
  int64_t bad = E;  // first edge with an out-of-range sender id
#pragma omp parallel for schedule(static) reduction(min : bad)
  for (int64_t e = 0; e < E; ++e)
    if (in.col[e] < 0 || in.col[e] >= n) bad = std::min(bad, e);
  if (bad < E) {
    char b[128];
    snprintf(b, sizeof b, "make_plan: sender id %d out of range at edge %lld", in.col[bad], (long long)bad);
    *err = b;
    return false;
  }
  if (E > INT32_MAX) {
    *err = "make_plan: more than 2^31-1 edges";
    return false;
  }
  if (in.sync_mode == kSyncGather) return make_gather_plan(in, out, err);
  if (in.sync_mode == kSyncTiledGather) return make_tgather_plan(in, out, err);
  if (in.sync_mode == kSyncBits) return make_bits_plan(in, out, err);
  // dense rows with one conductance whose edges cannot stay resident in shared
  // memory (2 bytes per edge per CTA): no stamped plan is possible, and auto
  // mode would pick the bitmask plan after building the tile plan; build it
  // directly
  if (in.sync_mode == kSyncAuto && !in.g && E * kBitsMinDensityInv >= (int64_t)n * (int64_t)n &&
      (E / std::max(1, in.grid_max)) * (int64_t)sizeof(uint16_t) > (int64_t)in.smem_budget)
    return make_bits_plan(in, out, err);
  const int threads = in.threads;
  const int nwarps = threads / 32;
  const int n_pad = pad_cells(n);

  // ---- grid size: enough CTAs that every warp gets about two chunks, and
  // for small networks at least min(n / 10, 100) CTAs: a stamped step is
  // latency-bound, and fewer cells per CTA shorten its gate units (one unit
  // per warp up to 32 cells), coupling and voltage step.  Measured per step
  // with Kahan sums: 1,000 cells at p = 0.1 (25 CTAs by the chunk count) 2.53
  // -> 1.95 us with 100 CTAs (2.20 with 152); 500 cells at p = 0.1 (7 CTAs)
  // 2.64 -> 1.85 us with 50; 2,000 cells at p = 0.02 (20 CTAs) 3.32 -> 2.18
  // us with 152; at p = 0.1 (98 CTAs) 152 CTAs were slower (2.52 against
  // 2.39 us), hence the cap at 100
  int grid = in.grid;
  if (grid <= 0) {
    const int64_t per_cta = (int64_t)nwarps * kChunkEdges * 2;
    grid = (int)std::min<int64_t>(in.grid_max, std::max<int64_t>(1, (E + per_cta - 1) / per_cta));
    grid = std::max(grid, std::min({in.grid_max, (n + 9) / 10, kSmallNetworkCtas}));
    grid = std::max(grid, (n + threads - 1) / threads);
  }
  grid = std::min(grid, in.grid_max);
  if ((int64_t)grid * threads < n) {
    *err = "make_plan: network larger than the co-resident thread count";
    return false;
  }
  std::vector<int> starts = in.cta_starts ? std::vector<int>(in.cta_starts, in.cta_starts + grid + 1)
                                          : partition_cells(n, in.row_ptr, grid, threads);
  const int ctas = (int)starts.size() - 1;
  int cells_cap = 32;
  for (int b = 0; b < ctas; ++b) cells_cap = std::max(cells_cap, ((starts[b + 1] - starts[b] + 31) / 32) * 32);

  // ---- per-CTA sorted edges (sender, g) and unique sender lists
  std::vector<std::vector<int>> uniq(ctas);
  int max_window = 4;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : max_window)
  for (int b = 0; b < ctas; ++b) {
    std::vector<int>& u = uniq[b];
    u.reserve((size_t)(in.row_ptr[starts[b + 1]] - in.row_ptr[starts[b]]));
    for (int c = starts[b]; c < starts[b + 1]; ++c)
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) u.push_back(in.col[e]);
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    if (!u.empty()) max_window = std::max(max_window, ((u.back() + 4) & ~3) - (u.front() & ~3));
  }

  // ---- tile capacity: one buffer holding the whole window when it fits,
  // otherwise two buffers for overlapped staging; shrink until smem fits.
  // chunk length: kChunkEdges, doubled while the partial-sum slots crowd out
  // the tiles
  int chunk = kChunkEdges;
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
        s += (cnt + chunk - 1) / chunk;
      }
    }
    return s;
  };
  int nbuf = 1, tile_cap = std::min(max_window, 65536);
  std::vector<std::vector<TileSpan>> tiles(ctas);
  int max_slots = 0;
  for (int attempt = 0; attempt < 32; ++attempt) {
    if (max_window > tile_cap) nbuf = 2;
    max_slots = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : max_slots)
    for (int b = 0; b < ctas; ++b) {
      tiles[b] = make_tiles(uniq[b], tile_cap, n_pad);
      max_slots = std::max(max_slots, slots_for(b, tiles[b]));
    }
    max_slots = std::max(max_slots, 1);
    if (plan_smem_bytes(tile_cap, nbuf, threads, cells_cap, max_slots, in.kahan) <= in.smem_budget) break;
    // slots taking over half of the budget: longer chunks first
    if (plan_smem_bytes(0, 0, threads, cells_cap, max_slots, in.kahan) * 2 > in.smem_budget &&
        chunk < kMaxChunkEdges) {
      chunk *= 2;
      continue;
    }
    // shrink: give the tiles what is left after the fixed part
    size_t fixed = plan_smem_bytes(0, 0, threads, cells_cap, max_slots, in.kahan);
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
  if (plan_smem_bytes(tile_cap, nbuf, threads, cells_cap, max_slots, in.kahan) > in.smem_budget) {
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
  P.smem_bytes = plan_smem_bytes(tile_cap, nbuf, threads, cells_cap, max_slots, in.kahan);
  P.cell_slots.assign(n, CellSlots{0, 0});
  // Each CTA's tables are built on their own (in parallel, indices local to
  // the CTA), then concatenated in CTA order with their offsets applied.
  struct Local {
    std::vector<TileDesc> tiles;
    std::vector<ChunkDesc> chunks;
    std::vector<uint16_t> edges;
    std::vector<float> edge_g;
    int n_slots = 0;
  };
  std::vector<Local> loc(ctas);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < ctas; ++b) {
    Local& L = loc[b];
    const std::vector<TileSpan>& tl = tiles[b];
    // senders of the CTA's cells, each cell's sorted by id, end to end
    std::vector<std::pair<int, float>> snd;
    snd.reserve((size_t)(in.row_ptr[starts[b + 1]] - in.row_ptr[starts[b]]));
    struct Pending {
      int tile, recv, slot;
      size_t begin, count;  // range in snd
    };
    std::vector<Pending> pend;
    int slot = 0;
    for (int c = starts[b]; c < starts[b + 1]; ++c) {
      const int r = c - starts[b];
      const size_t s0 = snd.size();
      for (int64_t e = in.row_ptr[c]; e < in.row_ptr[c + 1]; ++e) snd.push_back({in.col[e], in.g ? in.g[e] : 0.0f});
      std::stable_sort(snd.begin() + s0, snd.end(),
                       [](const std::pair<int, float>& x, const std::pair<int, float>& y) { return x.first < y.first; });
      P.cell_slots[c].begin = slot;
      size_t k = s0;
      for (int j = 0; j < (int)tl.size(); ++j) {
        const size_t t0 = k;
        while (k < snd.size() && snd[k].first < tl[j].hi) ++k;
        for (size_t o = t0; o < k; o += chunk) pend.push_back({j, r, slot++, o, std::min(k - o, (size_t)chunk)});
      }
      P.cell_slots[c].count = slot - P.cell_slots[c].begin;
    }
    L.n_slots = slot;
    // tile-major; inside a tile, larger chunks first (round-robin to warps)
    std::stable_sort(pend.begin(), pend.end(), [](const Pending& x, const Pending& y) {
      if (x.tile != y.tile) return x.tile < y.tile;
      return x.count > y.count;
    });
    L.edges.reserve(snd.size());
    if (in.g) L.edge_g.reserve(snd.size());
    size_t pi = 0;
    for (int j = 0; j < (int)tl.size(); ++j) {
      TileDesc td{};
      td.lo = tl[j].lo;
      td.nfloats = tl[j].hi - tl[j].lo;
      td.chunk_begin = (int)L.chunks.size();
      while (pi < pend.size() && pend[pi].tile == j) {
        const Pending& pc = pend[pi++];
        ChunkDesc cd{};
        cd.edge_begin = (int)L.edges.size();
        cd.slot = pc.slot;
        cd.recv = pc.recv;
        cd.count = (int)pc.count;
        for (size_t q = pc.begin; q < pc.begin + pc.count; ++q) {
          L.edges.push_back((uint16_t)(snd[q].first - td.lo));
          if (in.g) L.edge_g.push_back(snd[q].second);
        }
        L.chunks.push_back(cd);
      }
      td.chunk_end = (int)L.chunks.size();
      L.tiles.push_back(td);
    }
  }
  P.edges.reserve(E);
  if (in.g) P.edge_g.reserve(E);
  int slot_base = 0;
  for (int b = 0; b < ctas; ++b) {
    Local& L = loc[b];
    CtaWork w{};
    w.cell_begin = starts[b];
    w.n_cells = starts[b + 1] - starts[b];
    w.tile_begin = (int)P.tiles.size();
    w.n_tiles = (int)L.tiles.size();
    w.slot_begin = slot_base;
    w.n_slots = L.n_slots;
    const int chunk0 = (int)P.chunks.size(), edge0 = (int)P.edges.size();
    for (TileDesc td : L.tiles) {
      td.chunk_begin += chunk0;
      td.chunk_end += chunk0;
      P.tiles.push_back(td);
    }
    for (ChunkDesc cd : L.chunks) {
      cd.edge_begin += edge0;
      P.chunks.push_back(cd);
    }
    P.edges.insert(P.edges.end(), L.edges.begin(), L.edges.end());
    if (in.g) P.edge_g.insert(P.edge_g.end(), L.edge_g.begin(), L.edge_g.end());
    slot_base += L.n_slots;
    P.cta.push_back(w);
    std::vector<TileDesc>().swap(L.tiles);
    std::vector<ChunkDesc>().swap(L.chunks);
    std::vector<uint16_t>().swap(L.edges);
    std::vector<float>().swap(L.edge_g);
  }

  // ---- shared-memory shape; keep the static work resident when it fits
  SmemShape sh{};
  sh.tile_cap = tile_cap;
  sh.nbuf = nbuf;
  sh.threads = threads;
  sh.cells_cap = cells_cap;
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

  // ---- stamped exchange when every CTA's window (its unique senders, one
  // word each) fits in shared memory at once
  if (in.sync_mode != kSyncBarrier) {
    int sum_max = 4;
    for (int b = 0; b < ctas; ++b) sum_max = std::max(sum_max, (int)uniq[b].size());
    // stamped plans keep their work resident in the packed lane-chunk layout,
    // 16-bit byte offsets from the start of dynamic shared memory (so every
    // offset must stay below 64 KiB)
    // Preferred: two copies of the window, the second 16 banks away, so every
    // gather can pick the copy whose bank is free; else a single copy.
    SmemShape st = sh;
    Plan packed;
    bool fits = false;
    for (int dup = 1; dup >= 0 && !fits; --dup) {
      st = sh;
      st.nbuf = 1;
      st.stamped = 1;
      const int w4 = (sum_max + 3) & ~3;
      st.dup_words = dup ? ((w4 + 31) & ~31) + 16 : 0;
      st.tile_cap = dup ? st.dup_words + w4 : w4;
      const SmemLayout SL0 = smem_layout(st);  // tile and cell-array offsets do not depend on the rest
      const bool offsets_fit = SL0.vown + sizeof(float) * (size_t)(kScaledVArray + 1) * cells_cap <= 65536;
      if (in.no_resident || !offsets_fit) continue;
      packed = P;
      pack_groups(packed, SL0, in, uniq, st.dup_words, cells_cap);
      int mg = 1;
      for (const CtaWork& w : packed.cta) mg = std::max(mg, w.n_groups);
      st.max_slots = packed.max_slots;
      st.res_tiles = (sum_max + 3) / 4;  // the window's cell ids, four per 16-byte descriptor slot
      st.res_chunks = mg * 32;
      st.res_edges = mg * kGroupEntries;
      fits = smem_layout(st).total <= in.smem_budget;
    }
    if (fits) {
      sh = st;
      P.cta.swap(packed.cta);
      P.cell_slots.swap(packed.cell_slots);
      P.gdesc.swap(packed.gdesc);
      P.edges.swap(packed.edges);
      P.edge_g.swap(packed.edge_g);
      P.max_slots = packed.max_slots;
      // the windows replace the tiles: CTA b's window is gcol[tile_begin ..
      // tile_begin + n_tiles), its unique senders in ascending order
      P.tiles.clear();
      P.chunks.clear();
      P.gcol.clear();
      for (int b = 0; b < ctas; ++b) {
        CtaWork& w = P.cta[b];
        w.tile_begin = (int)P.gcol.size();
        w.n_tiles = (int)uniq[b].size();
        P.gcol.insert(P.gcol.end(), uniq[b].begin(), uniq[b].end());
      }
      // progress probes: CTAs that read a CTA's cells without being read by it
      std::vector<int> owner(n);
      for (int b = 0; b < ctas; ++b)
        for (int c = starts[b]; c < starts[b + 1]; ++c) owner[c] = b;
      std::vector<std::vector<char>> reads(ctas, std::vector<char>(ctas, 0));  // reads[r][x]: r polls x
      for (int b = 0; b < ctas; ++b)
        for (int c : uniq[b]) reads[b][owner[c]] = 1;
      for (int x = 0; x < ctas; ++x) {
        CtaWork& w = P.cta[x];
        w.probe_begin = (int)P.probes.size();
        for (int r = 0; r < ctas; ++r)
          if (r != x && reads[r][x] && !reads[x][r]) P.probes.push_back(starts[r]);
        w.n_probes = (int)P.probes.size() - w.probe_begin;
      }
      sh.poll_words = 0;
      for (const CtaWork& w : P.cta) sh.poll_words = std::max(sh.poll_words, w.n_tiles + w.n_probes);
    } else if (in.sync_mode == kSyncStamped) {
      *err = "make_plan: stamped exchange requested but the tiles do not fit in shared memory";
      return false;
    }
  }
  P.shape = sh;
  P.smem_bytes = smem_layout(sh).total;
  // windows larger than shared memory and short rows: gather through L2
  // instead of staging tiles (each row would be cut into a few edges per tile)
  // windows larger than shared memory: dense rows with one conductance walk
  // adjacency bits; short rows gather through staged tiles
  if (!sh.stamped && in.sync_mode == kSyncAuto && !in.g &&
      E * kBitsMinDensityInv >= (int64_t)n * (int64_t)n)
    return make_bits_plan(in, out, err);
  if (!sh.stamped && in.sync_mode == kSyncAuto && E <= (int64_t)kGatherMaxMeanDegree * n)
    return make_tgather_plan(in, out, err);
  return true;
}

namespace {

uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations:
// eigenvalues in w, eigenvectors in the columns of V.
void jacobi3(double A[3][3], double w[3], double V[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    if (off < 1e-30) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (std::fabs(A[p][q]) < 1e-300) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; ++k) {  // A <- A J
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {  // A <- J^T A
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

int max_window(const Plan& P) {
  int m = 0;
  for (const CtaWork& w : P.cta) m = std::max(m, w.n_tiles);
  return m;
}

}  // namespace

// Spectral coordinates: the two lowest non-trivial eigenvectors of the
// in-edge graph Laplacian L = D - A (D = in-degrees), by subspace iteration
// with three vectors on (c I - L), c = 2 max degree + 1, deflating the
// constant vector every step, then a Rayleigh-Ritz step.  On graphs whose
// edges join nearby cells (distance-dependent connectivity) these
// coordinates follow the cells' positions.  Recursive coordinate bisection
// of them (along the wider extent, balanced by the planner's CTA cost) gives
// `parts` compact blocks; cells keep ascending ids inside a block.
std::vector<int> locality_order(const PlanInput& in, int parts, int threads, std::vector<int>* starts) {
  const int n = in.n;
  std::vector<int> order;
  if (n < 8 || parts < 2 || (int64_t)parts * threads < n) return order;
  double dmax = 0.0;
  for (int i = 0; i < n; ++i) dmax = std::max(dmax, (double)(in.row_ptr[i + 1] - in.row_ptr[i]));
  const double cshift = 2.0 * dmax + 1.0;
  std::vector<double> X((size_t)n * 3), Y((size_t)n * 3);
  uint64_t rs = 0x5eed5eedull;
  for (double& x : X) x = (double)(splitmix64(&rs) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  auto deflate = [&](std::vector<double>& M) {
    for (int k = 0; k < 3; ++k) {
      double m = 0.0;
      for (int i = 0; i < n; ++i) m += M[(size_t)i * 3 + k];
      m /= n;
      for (int i = 0; i < n; ++i) M[(size_t)i * 3 + k] -= m;
    }
  };
  auto apply_L = [&](const std::vector<double>& Xi, std::vector<double>& Yo, double shift) {
    // Yo = shift * Xi - L Xi
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double s0 = 0.0, s1 = 0.0, s2 = 0.0;
      for (int64_t e = in.row_ptr[i]; e < in.row_ptr[i + 1]; ++e) {
        const size_t j = (size_t)in.col[e] * 3;
        s0 += Xi[j];
        s1 += Xi[j + 1];
        s2 += Xi[j + 2];
      }
      const double d = (double)(in.row_ptr[i + 1] - in.row_ptr[i]);
      const size_t o = (size_t)i * 3;
      Yo[o] = shift * Xi[o] - (d * Xi[o] - s0);
      Yo[o + 1] = shift * Xi[o + 1] - (d * Xi[o + 1] - s1);
      Yo[o + 2] = shift * Xi[o + 2] - (d * Xi[o + 2] - s2);
    }
  };
  auto orthonormalize = [&](std::vector<double>& M) {
    for (int k = 0; k < 3; ++k) {
      for (int q = 0; q < k; ++q) {
        double dot = 0.0;
        for (int i = 0; i < n; ++i) dot += M[(size_t)i * 3 + k] * M[(size_t)i * 3 + q];
        for (int i = 0; i < n; ++i) M[(size_t)i * 3 + k] -= dot * M[(size_t)i * 3 + q];
      }
      double nrm = 0.0;
      for (int i = 0; i < n; ++i) nrm += M[(size_t)i * 3 + k] * M[(size_t)i * 3 + k];
      nrm = std::sqrt(nrm);
      if (nrm < 1e-300) return false;
      for (int i = 0; i < n; ++i) M[(size_t)i * 3 + k] /= nrm;
    }
    return true;
  };
  deflate(X);
  if (!orthonormalize(X)) return order;
  for (int it = 0; it < kReorderIters; ++it) {
    apply_L(X, Y, cshift);
    deflate(Y);
    if (!orthonormalize(Y)) return order;
    X.swap(Y);
  }
  // Rayleigh-Ritz: H = X^T L X (Y = -L X with shift 0)
  apply_L(X, Y, 0.0);
  double H[3][3], w[3], V[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double h = 0.0;
      for (int i = 0; i < n; ++i) h -= X[(size_t)i * 3 + a] * Y[(size_t)i * 3 + b];
      H[a][b] = h;
    }
  for (int a = 0; a < 3; ++a)
    for (int b = a + 1; b < 3; ++b) H[a][b] = H[b][a] = 0.5 * (H[a][b] + H[b][a]);
  jacobi3(H, w, V);
  int idx[3] = {0, 1, 2};
  std::sort(idx, idx + 3, [&](int p, int q) { return w[p] < w[q]; });
  std::vector<double> C((size_t)n * 2);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 2; ++k) {
      double v = 0.0;
      for (int a = 0; a < 3; ++a) v += X[(size_t)i * 3 + a] * V[a][idx[k]];
      C[(size_t)i * 2 + k] = v;
    }
  // recursive coordinate bisection, balanced by the CTA cost
  std::vector<int64_t> cost(n);
  for (int i = 0; i < n; ++i) cost[i] = (in.row_ptr[i + 1] - in.row_ptr[i]) + kCellCost;
  std::vector<int> ids(n);
  for (int i = 0; i < n; ++i) ids[i] = i;
  order.reserve(n);
  starts->assign(1, 0);
  struct Range {
    int lo, hi, parts;
  };
  std::vector<Range> stack{{0, n, parts}};
  while (!stack.empty()) {
    const Range r = stack.back();
    stack.pop_back();
    if (r.parts == 1 || r.hi - r.lo <= 1) {
      if (r.hi - r.lo > threads) {
        order.clear();
        return order;
      }
      std::sort(ids.begin() + r.lo, ids.begin() + r.hi);
      order.insert(order.end(), ids.begin() + r.lo, ids.begin() + r.hi);
      starts->push_back((int)order.size());
      // a leaf of several parts with one cell: the remaining parts stay empty
      continue;
    }
    double lo0 = 1e300, hi0 = -1e300, lo1 = 1e300, hi1 = -1e300;
    for (int k = r.lo; k < r.hi; ++k) {
      const double* c = &C[(size_t)ids[k] * 2];
      lo0 = std::min(lo0, c[0]);
      hi0 = std::max(hi0, c[0]);
      lo1 = std::min(lo1, c[1]);
      hi1 = std::max(hi1, c[1]);
    }
    const int ax = (hi0 - lo0) >= (hi1 - lo1) ? 0 : 1;
    std::stable_sort(ids.begin() + r.lo, ids.begin() + r.hi, [&](int p, int q) {
      const double a = C[(size_t)p * 2 + ax], b = C[(size_t)q * 2 + ax];
      return a < b || (a == b && p < q);
    });
    const int p1 = r.parts / 2;
    int64_t total = 0;
    for (int k = r.lo; k < r.hi; ++k) total += cost[ids[k]];
    const double target = (double)total * p1 / r.parts;
    int64_t acc = 0;
    int cut = r.lo;
    while (cut < r.hi - 1 && (double)(acc + cost[ids[cut]]) <= target) acc += cost[ids[cut++]];
    if (cut == r.lo) ++cut;
    // second half pushed first, so the first half is emitted first
    stack.push_back({cut, r.hi, r.parts - p1});
    stack.push_back({r.lo, cut, p1});
  }
  if ((int)order.size() != n) order.clear();
  return order;
}

// Plans the network as given; for stamped plans with wide windows, also
// plans it in a locality-preserving cell order and keeps that plan when its
// largest window is at least a fifth smaller.
bool make_plan(const PlanInput& in, Plan* out, std::string* err) {
  if (!make_plan_base(in, out, err)) return false;
  if (!in.reorder || in.cta_starts || !out->shape.stamped || out->cta.size() < 2) return true;
  const int n = in.n;
  const int ctas = (int)out->cta.size();
  const int64_t E = in.row_ptr[n];
  const int w0 = max_window(*out);
  const int per_cta = (n + ctas - 1) / ctas;
  if (E > kReorderMaxEdges || w0 > n / 2 || w0 < kReorderMinWindowRatio * per_cta) return true;
  std::vector<int> starts;
  std::vector<int> order = locality_order(in, ctas, in.threads, &starts);
  if (order.empty() || (int)starts.size() != ctas + 1) return true;
  std::vector<int> inv(n);
  for (int i = 0; i < n; ++i) inv[order[i]] = i;
  std::vector<int64_t> rp(n + 1, 0);
  std::vector<int32_t> col((size_t)E);
  std::vector<float> g(in.g ? (size_t)E : 0);
  for (int r = 0; r < n; ++r) rp[r + 1] = rp[r] + (in.row_ptr[order[r] + 1] - in.row_ptr[order[r]]);
#pragma omp parallel for schedule(dynamic, 64)
  for (int r = 0; r < n; ++r) {
    const int o = order[r];
    std::vector<std::pair<int, float>> e;
    e.reserve((size_t)(in.row_ptr[o + 1] - in.row_ptr[o]));
    for (int64_t k = in.row_ptr[o]; k < in.row_ptr[o + 1]; ++k) e.push_back({inv[in.col[k]], in.g ? in.g[k] : 0.0f});
    std::stable_sort(e.begin(), e.end(),
                     [](const std::pair<int, float>& x, const std::pair<int, float>& y) { return x.first < y.first; });
    for (size_t k = 0; k < e.size(); ++k) {
      col[(size_t)rp[r] + k] = e[k].first;
      if (in.g) g[(size_t)rp[r] + k] = e[k].second;
    }
  }
  PlanInput in2 = in;
  in2.row_ptr = rp.data();
  in2.col = col.data();
  in2.g = in.g ? g.data() : nullptr;
  in2.grid = ctas;
  in2.cta_starts = starts.data();
  Plan P2;
  std::string e2;
  if (!make_plan_base(in2, &P2, &e2) || !P2.shape.stamped || (int)P2.cta.size() != ctas) return true;
  if ((int64_t)max_window(P2) * 5 > (int64_t)w0 * 4) return true;
  P2.perm.assign(order.begin(), order.end());
  *out = std::move(P2);
  return true;
}

}  // namespace infoli

// ---------------------------------------------------------------------------
// Host emulation of a plan: plans a network exactly as infoli_sim_create
// would for the given launch limits, then evaluates the gap-junction
// currents by walking the plan's tables with the step kernel's addressing
// (tile staging, byte offsets into the shared-memory image, padding entries,
// partial slots).  Every shared-memory offset is bounds-checked.  Used by the
// CPU test suite to validate the planner without a GPU.
extern "C" int infoli_plan_emulate(int n, const int64_t* row_ptr, const int32_t* col, const float* g,
                                   float g_uniform, int grid, int grid_max, int threads, int64_t smem_budget,
                                   int sync_mode, const float* vdend_in, float* ic_out_in, int64_t info[10]) {
  using namespace infoli;
  PlanInput in;
  in.n = n;
  in.row_ptr = row_ptr;
  in.col = col;
  in.g = g;
  in.grid = grid;
  in.grid_max = grid_max;
  in.threads = threads;
  in.smem_budget = (size_t)smem_budget;
  in.sync_mode = sync_mode;
  Plan P;
  std::string err;
  if (!make_plan(in, &P, &err)) return -1;
  // relabelled plans: evaluate in plan order, report in the caller's order
  std::vector<float> v_plan, ic_plan;
  const float* vdend = vdend_in;
  float* ic_out = ic_out_in;
  if (!P.perm.empty()) {
    if ((int)P.perm.size() != n) return -9;
    std::vector<char> seen(n, 0);
    v_plan.resize(n);
    ic_plan.assign(n, 0.0f);
    for (int i = 0; i < n; ++i) {
      const int o = P.perm[i];
      if (o < 0 || o >= n || seen[o]) return -9;
      seen[o] = 1;
      v_plan[i] = vdend_in[o];
    }
    vdend = v_plan.data();
    ic_out = ic_plan.data();
  }
  const SmemLayout L = smem_layout(P.shape);
  if (P.shape.gather >= 2 ? tgather_smem_bytes(P.shape) > (size_t)smem_budget
                          : !P.shape.gather && L.total > (size_t)smem_budget)
    return -2;
  auto fexp = [](float V) { return 0.8f * std::exp(-(V * V) / 100.0f) + 0.2f; };
  std::vector<unsigned char> sm(P.shape.gather ? 0 : L.total);
  int64_t groups = 0, probes = 0, gather_waves = 0, gathers = 0;
  for (const CtaWork& w : P.cta) {
    if (w.n_cells > threads || w.n_cells > P.shape.cells_cap) return -3;
    if (P.shape.gather == 3) {
      const int wpr = w.pad0;
      for (int t = 0; t < w.n_cells; ++t) {
        const int c = w.cell_begin + t;
        float acc = 0.0f;
        for (int j = 0; j < w.n_tiles; ++j) {
          const TileDesc& td = P.tiles[w.tile_begin + j];
          if (td.lo != td.chunk_begin * 32 || td.nfloats > P.shape.tile_cap || td.lo % 32) return -4;
          for (int col = td.chunk_begin; col < td.chunk_end; ++col) {
            const size_t at = (size_t)w.slot_begin + (size_t)col * w.n_cells + t;
            if (col >= wpr || at >= P.gcol.size()) return -8;
            const uint32_t x = (uint32_t)P.gcol[at];
            for (int k = 0; k < 32; ++k)
              if (x & (0x80000000u >> k)) {
                const int s = col * 32 + k;
                if (s >= n || s - td.lo >= td.nfloats) return -7;
                const float V = vdend[c] - vdend[s];
                acc += fexp(V) * V;
              }
          }
        }
        ic_out[c] = acc * g_uniform;
      }
      continue;
    }
    if (P.shape.gather == 2) {
      if (P.smem_bytes < tgather_smem_bytes(P.shape)) return -2;
      for (int t = 0; t < w.n_cells; ++t) {
        const int c = w.cell_begin + t;
        float acc = 0.0f;
        for (int j = 0; j < w.n_tiles; ++j) {
          const TileDesc& td = P.tiles[w.tile_begin + j];
          if (td.lo < 0 || td.lo % 4 || td.nfloats % 4 || td.nfloats > P.shape.tile_cap) return -4;
          const size_t ci = (size_t)w.slot_begin + (size_t)j * w.n_cells + t;
          if (ci >= P.gcol.size()) return -8;
          const int cnt = P.gcol[ci];
          if (cnt < 0 || cnt > td.chunk_end) return -8;
          for (int k = 0; k < cnt; ++k) {
            const size_t at = (size_t)td.chunk_begin + (size_t)k * w.n_cells + t;
            if (at >= P.edges.size()) return -8;
            const int o = P.edges[at];
            if (o >= td.nfloats || td.lo + o >= n) return -7;
            const float V = vdend[c] - vdend[td.lo + o];
            acc += (g ? P.edge_g[at] : 1.0f) * fexp(V) * V;
          }
        }
        ic_out[c] = g ? acc : acc * g_uniform;
      }
      continue;
    }
    if (P.shape.gather) {
      for (int t = 0; t < w.n_cells; ++t) {
        const int c = w.cell_begin + t;
        float acc = 0.0f;
        for (int j = 0; j < w.pad0; ++j) {
          const size_t at = (size_t)w.slot_begin + (size_t)j * w.n_cells + t;
          if (at >= P.gcol.size()) return -8;
          const int s = P.gcol[at];
          if (s < 0 || s >= n) return -7;
          const float V = vdend[c] - vdend[s];
          acc += (g ? P.edge_g[at] : 1.0f) * fexp(V) * V;
        }
        ic_out[c] = g ? acc : acc * g_uniform;
      }
      continue;
    }
    std::fill(sm.begin(), sm.end(), 0);
    float* fsm = reinterpret_cast<float*>(sm.data());
    std::vector<float> part(P.shape.max_slots, 0.0f);
    float* sVd = reinterpret_cast<float*>(sm.data() + L.vown);
    for (int r = 0; r < w.n_cells; ++r) sVd[r] = vdend[w.cell_begin + r];
    // stamped plans' padding entries read the scaled-V array; the emulation
    // runs unscaled, so it holds the plain V_dend here
    for (int r = 0; r < w.n_cells; ++r) sVd[(size_t)kScaledVArray * P.shape.cells_cap + r] = vdend[w.cell_begin + r];
    if (P.shape.stamped) {
      // the window: the CTA's unique senders, one float each (and the
      // bank-shifted second copy), ids held four per descriptor slot
      const size_t dup = (size_t)P.shape.dup_words;
      const size_t nw = (size_t)w.n_tiles;
      if (w.tile_begin < 0 || (size_t)w.tile_begin + nw > P.gcol.size() || dup + nw > (size_t)P.shape.tile_cap ||
          (dup && nw > dup) || nw > (size_t)P.shape.res_tiles * 4)
        return -4;
      for (size_t i = 0; i < nw; ++i) {
        const int c = P.gcol[(size_t)w.tile_begin + i];
        if (c < 0 || c >= n || (i > 0 && c <= P.gcol[(size_t)w.tile_begin + i - 1])) return -4;
        fsm[i] = vdend[c];
        if (dup) fsm[dup + i] = fsm[i];
      }
      for (int q = 0; q < w.n_probes; ++q)
        if (P.probes[w.probe_begin + q] < 0 || P.probes[w.probe_begin + q] >= n) return -5;
      probes += w.n_probes;
      groups += w.n_groups;
      // shared-memory wavefronts of the V_dend gathers: per (group, entry
      // position) the largest number of distinct words any bank serves
      for (int gi = 0; gi < w.n_groups; ++gi)
        for (int k = 0; k < kLaneEdges; ++k) {
          unsigned words[32][32];
          int cnt[32] = {0};
          int worst = 1;
          for (int l = 0; l < 32; ++l) {
            const size_t at = (((size_t)w.group_begin + gi) * kQuads + k / 4) * 32 * 4 + (size_t)l * 4 + k % 4;
            const unsigned word = P.edges[at] >> 2, bank = word & 31;
            bool seen = false;
            for (int q = 0; q < cnt[bank]; ++q) seen |= words[bank][q] == word;
            if (!seen) words[bank][cnt[bank]++] = word;
            worst = std::max(worst, cnt[bank]);
          }
          gather_waves += worst;
          gathers += 1;
        }
      for (int gi = 0; gi < w.n_groups; ++gi)
        for (int l = 0; l < 32; ++l) {
          const int2_t d = P.gdesc[((size_t)w.group_begin + gi) * 32 + l];
          if (d.x < 0 || d.x >= P.shape.max_slots || d.y < 0 || d.y >= std::max(w.n_cells, 1)) return -6;
          const float vc = sVd[d.y];
          float acc0 = 0.0f, acc1 = 0.0f;
          for (int k = 0; k < kLaneEdges; ++k) {
            const size_t at = (((size_t)w.group_begin + gi) * kQuads + k / 4) * 32 * 4 + (size_t)l * 4 + k % 4;
            const unsigned off = P.edges[at];
            if (off % 4 || off + 4 > L.vown + sizeof(float) * (size_t)(kScaledVArray + 1) * P.shape.cells_cap) return -7;
            const float V = vc - *reinterpret_cast<const float*>(sm.data() + off);
            const float gg = g ? P.edge_g[at] : 1.0f;
            ((k & 1) ? acc1 : acc0) += (gg * fexp(V)) * V;
          }
          part[d.x] = acc0 + acc1;
        }
    } else {
      for (int j = 0; j < w.n_tiles; ++j) {
        const TileDesc& td = P.tiles[w.tile_begin + j];
        if (td.lo < 0 || td.lo % 4 || td.nfloats % 4 || td.nfloats > P.shape.tile_cap) return -4;
        for (int ci = td.chunk_begin; ci < td.chunk_end; ++ci) {
          const ChunkDesc& c = P.chunks[ci];
          if (c.slot < 0 || c.slot >= P.shape.max_slots || c.recv < 0 || c.recv >= w.n_cells) return -6;
          float acc = 0.0f;
          for (int k = 0; k < c.count; ++k) {
            const int o = P.edges[c.edge_begin + k];
            if (o >= td.nfloats || td.lo + o >= n) return -7;
            const float V = sVd[c.recv] - vdend[td.lo + o];
            acc += (g ? P.edge_g[c.edge_begin + k] : 1.0f) * fexp(V) * V;
          }
          part[c.slot] = acc;
        }
      }
      groups += P.tiles.empty() ? 0 : 0;
    }
    for (int r = 0; r < w.n_cells; ++r) {
      const CellSlots cs = P.cell_slots[w.cell_begin + r];
      float ic = 0.0f;
      for (int q = 0; q < cs.count; ++q) ic += part[cs.begin + q];
      ic_out[w.cell_begin + r] = g ? ic : ic * g_uniform;
    }
  }
  if (!P.perm.empty())
    for (int i = 0; i < n; ++i) ic_out_in[P.perm[i]] = ic_plan[i];
  if (info) {
    info[0] = P.grid;
    info[1] = P.shape.gather ? 1 + P.shape.gather : P.shape.stamped;
    info[2] = P.shape.stamped ? (int64_t)!P.perm.empty() : (int64_t)P.tiles.size();
    info[3] = P.shape.stamped ? groups : (int64_t)P.chunks.size();
    info[4] = P.shape.max_slots;
    info[5] = (int64_t)P.smem_bytes;
    info[6] = probes;
    info[7] = P.shape.res_chunks > 0;
    info[8] = gather_waves;
    info[9] = gathers;
  }
  return 0;
}

// The planner's locality-preserving cell order (see locality_order): order[new]
// = old cell, starts = the CTA ranges in the new order (parts + 1 entries).
// Returns 0, or -1 when no order was found.
extern "C" int infoli_plan_locality_order(int n, const int64_t* row_ptr, const int32_t* col, int parts,
                                          int threads, int32_t* order_out, int32_t* starts_out) {
  using namespace infoli;
  if (n <= 0 || !row_ptr || (row_ptr[n] > 0 && !col) || parts < 1 || threads < 1 || !order_out || !starts_out)
    return -1;
  PlanInput in;
  in.n = n;
  in.row_ptr = row_ptr;
  in.col = col;
  std::vector<int> starts;
  const std::vector<int> order = locality_order(in, parts, threads, &starts);
  if ((int)order.size() != n || (int)starts.size() != parts + 1) return -1;
  for (int i = 0; i < n; ++i) order_out[i] = order[i];
  for (int i = 0; i <= parts; ++i) starts_out[i] = starts[i];
  return 0;
}
