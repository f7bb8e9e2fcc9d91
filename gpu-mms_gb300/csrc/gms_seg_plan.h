// Host plan of a segmented (batched) sort: many independent arrays
// ("segments") of uneven length, each sorted by its own base-case tiles and
// merge rounds, every round launched once over all segments.  Plain C++ (no
// CUDA), so the CPU tests compile and check it directly.
//
// No counterpart in the reference, which sorts one array per multimergesort
// call (GPU-MMS src/multimergesort.hxx:56-141): a batch there is a loop of
// calls, each running the round loop of multimergesort.hxx:87-135 for its own
// array.  Here one launch per round serves every array, and no group of a
// round crosses an array's end.
//
// Size classes fall out of the round count R_s = ceil(log_k(len_s / base)):
//   R_s = 0  the segment fits one base tile: sorted in one pass by the base
//            case, straight into the output;
//   R_s = 1  up to k base tiles: one merge round, its groups merged by one
//            CTA each when k * base fits a CTA, else cut into forecast tiles;
//   R_s > 1  rounds bounded to the segment: round p merges groups of k runs
//            of base * k^(p-1) keys inside the segment.
// A segment leaves the round loop after its R_s rounds.  Its buffers
// alternate between the output and a scratch array so that its last round
// (or its base case, when R_s = 0) writes the output: the base case writes
// B_0 and round p writes B_p, with B_q = output when R_s - q is even and the
// scratch array otherwise.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace gms {

// Engine constants the plan follows.
struct SegGeom {
  int64_t base_tile;             // keys of a base-case tile
  int64_t cap_data, capw_data;   // data rounds: keys one CTA merges whole / keys of a forecast tile
  int64_t cap_idx, capw_idx;     // the same for sample rounds (uint32 index payload)
  int k;                         // fan-in
  int sample_b;                  // block of the forecast sample
  int max_levels;                // deepest sample recursion the scratch layout holds
};

// Same layout as GroupDesc in gms_kernels.cuh.
struct SegGroupH {
  int64_t start, len, run0, tile0, row0, flags;
};
constexpr int64_t kSegAlt = 1;  // GRP_ALT: the second buffer pair
constexpr int64_t kSegDec = 2;  // GRP_DEC: decode keys on store

// One round at one recursion level.
struct SegLevelH {
  int depth = 0;                  // 0: a data round; d > 0: its d-th level of sample merges
  int64_t n = 0;                  // extent of the arrays the round reads and writes
  int64_t L = 0;                  // run length
  int64_t runs = 0;               // input runs, numbered globally over the round's producer
  bool whole = false;             // k * L fits a CTA: one CTA merges each group, no tiles
  std::vector<SegGroupH> grp;     // groups, then one entry with the totals
  std::vector<int32_t> tile_grp;  // group of every forecast tile
  std::vector<int32_t> row_grp;   // group of every boundary row
  std::vector<int32_t> run_len;   // length of every input run (gathers of the sample read it)
  int sample = -1;                // index in SegPlanH::levels of its sample merge (-1: none)
};

struct SegPlanH {
  int64_t n = 0;
  int rounds_max = 0;
  std::vector<SegGroupH> base;  // base-case tiles, one group (run) each
  std::vector<int> rounds;      // level index of data rounds 1 .. rounds_max
  std::vector<SegLevelH> levels;
  bool ok = true;
  bool too_long = false;  // an array longer than 2^31 - 1 keys (run lengths are 32-bit): no plan
  // scratch sizes in entries, as WsLayout: data-level block samples, gathered
  // samples and merged samples per level, boundary rows per level
  int64_t s1 = 0;
  int64_t s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t rows[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int depth = 0;
};

inline int64_t seg_ceil(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Merge rounds a segment of `len` keys needs after its base case.
inline int seg_rounds(int64_t len, int64_t base, int k) {
  int p = 0;
  for (int64_t L = base; L < len; L *= k) ++p;
  return p;
}

// Adds the level of one round (groups with start, len, run0 and flags set;
// runs of L keys, the last of a group possibly short) and, when its groups
// need forecast tiles, the levels of its sample merges.  Returns its index.
inline int seg_add_level(SegPlanH& P, const SegGeom& G, std::vector<SegGroupH> grp, int64_t n, int64_t L,
                         int64_t runs, bool idx, int depth) {
  const int at = (int)P.levels.size();
  P.levels.emplace_back();
  // (no single-letter names: callers of the drop-in header define the
  // reference's params.h macros K, B, M, W before including it)
  const int64_t k = G.k, blk = G.sample_b;
  const int64_t cap = idx ? G.cap_idx : G.cap_data;
  const int64_t capw = idx ? G.capw_idx : G.capw_data;
  const bool whole = k * L <= cap;
  std::vector<int32_t> tile_grp, row_grp, run_len((size_t)runs, 0);
  int64_t tile = 0, row = 0;
  const int64_t Ls = seg_ceil(L, blk);
  const int64_t Gt = capw / blk - k;  // sample entries between tile boundaries
  std::vector<SegGroupH> sgrp;
  for (size_t g = 0; g < grp.size(); ++g) {
    SegGroupH& h = grp[g];
    const int64_t kg = seg_ceil(h.len, L);
    const int64_t last = h.len - (kg - 1) * L;
    for (int64_t r = 0; r < kg; ++r) run_len[(size_t)(h.run0 + r)] = (int32_t)(r + 1 < kg ? L : last);
    h.tile0 = tile;
    h.row0 = row;
    if (!whole) {
      const int64_t ns = (kg - 1) * Ls + seg_ceil(last, blk);
      const int64_t tiles = seg_ceil(ns, Gt);
      tile_grp.insert(tile_grp.end(), (size_t)tiles, (int32_t)g);
      row_grp.insert(row_grp.end(), (size_t)(tiles + 1), (int32_t)g);
      tile += tiles;
      row += tiles + 1;
      sgrp.push_back(SegGroupH{h.run0 * Ls, ns, h.run0, 0, 0, 0});
    }
  }
  grp.push_back(SegGroupH{n, 0, runs, tile, row, 0});
  {
    SegLevelH& lv = P.levels[(size_t)at];
    lv.depth = depth;
    lv.n = n;
    lv.L = L;
    lv.runs = runs;
    lv.whole = whole;
    lv.grp = std::move(grp);
    lv.tile_grp = std::move(tile_grp);
    lv.row_grp = std::move(row_grp);
    lv.run_len = std::move(run_len);
  }
  if (!whole) {
    if (depth + 1 >= G.max_levels || Gt < 1) {
      P.ok = false;
      return at;
    }
    const int64_t ns_all = runs * Ls;  // the block samples of every run, Ls apart
    P.rows[depth] = std::max(P.rows[depth], row);
    P.f[depth + 1] = std::max(P.f[depth + 1], ns_all);
    if (depth == 0) {
      P.s1 = std::max(P.s1, ns_all);
    } else {
      P.s[depth + 1] = std::max(P.s[depth + 1], ns_all);
    }
    P.depth = std::max(P.depth, depth + 1);
    const int sub = seg_add_level(P, G, std::move(sgrp), ns_all, Ls, runs, true, depth + 1);
    P.levels[(size_t)at].sample = sub;
  }
  return at;
}

// The plan for segments [off[s], off[s+1]) of n = off[nseg] keys (off
// monotone, off[0] = 0; empty segments allowed).
inline SegPlanH seg_plan(const int64_t* off, int64_t nseg, const SegGeom& G) {
  SegPlanH P;
  P.n = nseg > 0 ? off[nseg] : 0;
  for (int64_t s = 0; s < nseg; ++s) {
    if (off[s + 1] - off[s] > (int64_t)0x7fffffff) {
      P.ok = false;
      P.too_long = true;
      return P;
    }
  }
  const int64_t k = G.k;
  std::vector<int> R((size_t)nseg, 0);
  std::vector<int64_t> first((size_t)nseg, 0), units((size_t)nseg, 0);
  for (int64_t s = 0; s < nseg; ++s) {
    const int64_t len = off[s + 1] - off[s];
    R[(size_t)s] = seg_rounds(len, G.base_tile, G.k);
    P.rounds_max = std::max(P.rounds_max, R[(size_t)s]);
    first[(size_t)s] = (int64_t)P.base.size();
    units[(size_t)s] = seg_ceil(len, G.base_tile);
    for (int64_t t = 0; t * G.base_tile < len; ++t) {
      const int64_t st = off[s] + t * G.base_tile;
      const int64_t fl = (R[(size_t)s] % 2 == 0 ? kSegAlt : 0) | (R[(size_t)s] == 0 ? kSegDec : 0);
      P.base.push_back(SegGroupH{st, std::min(G.base_tile, off[s + 1] - st), (int64_t)P.base.size(), 0, 0, fl});
    }
  }
  int64_t prev_units = (int64_t)P.base.size();
  int64_t L = G.base_tile;
  for (int p = 1; p <= P.rounds_max; ++p, L *= k) {
    std::vector<SegGroupH> grp;
    for (int64_t s = 0; s < nseg; ++s) {
      if (R[(size_t)s] < p) continue;
      const int64_t len = off[s + 1] - off[s];
      const int64_t m = units[(size_t)s];  // this segment's input runs
      const int64_t f0 = (int64_t)grp.size();
      for (int64_t q = 0; q * k < m; ++q) {
        const int64_t st = off[s] + q * L * k;
        const int64_t fl = ((R[(size_t)s] - p) % 2 ? kSegAlt : 0) | (R[(size_t)s] == p ? kSegDec : 0);
        grp.push_back(SegGroupH{st, std::min(L * k, off[s + 1] - st), first[(size_t)s] + q * k, 0, 0, fl});
      }
      (void)len;
      first[(size_t)s] = f0;
      units[(size_t)s] = (int64_t)grp.size() - f0;
    }
    const int64_t ng = (int64_t)grp.size();
    // the producers write the block samples of every run, Ls apart
    P.s1 = std::max(P.s1, prev_units * seg_ceil(L, G.sample_b));
    P.rounds.push_back(seg_add_level(P, G, std::move(grp), P.n, L, prev_units, false, 0));
    prev_units = ng;
  }
  return P;
}

// Byte layout of a plan's device arrays in one blob (256-byte aligned parts):
// the base tiles' groups, then per level its groups, tile and row maps and
// run lengths.
struct SegBlobLevel {
  size_t grp = 0, tile_grp = 0, row_grp = 0, run_len = 0;
};
struct SegBlob {
  size_t base = 0;
  std::vector<SegBlobLevel> lv;
  size_t bytes = 0;
};

inline SegBlob seg_blob_layout(const SegPlanH& P) {
  SegBlob b;
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t r = at;
    at += (bytes + 255) / 256 * 256;
    return r;
  };
  b.base = take(sizeof(SegGroupH) * (P.base.size() + 1));
  for (const SegLevelH& l : P.levels) {
    SegBlobLevel x;
    x.grp = take(sizeof(SegGroupH) * l.grp.size());
    x.tile_grp = take(sizeof(int32_t) * (l.tile_grp.size() + 1));
    x.row_grp = take(sizeof(int32_t) * (l.row_grp.size() + 1));
    x.run_len = take(sizeof(int32_t) * (l.run_len.size() + 1));
    b.lv.push_back(x);
  }
  b.bytes = at;
  return b;
}

// Fills `out` (b.bytes) with the plan's arrays at the layout's offsets.
inline void seg_blob_fill(const SegPlanH& P, const SegBlob& b, unsigned char* out) {
  auto put = [&](size_t off, const void* src, size_t bytes) {
    const unsigned char* c = static_cast<const unsigned char*>(src);
    std::copy(c, c + bytes, out + off);
  };
  std::fill(out, out + b.bytes, (unsigned char)0);
  put(b.base, P.base.data(), sizeof(SegGroupH) * P.base.size());
  for (size_t i = 0; i < P.levels.size(); ++i) {
    const SegLevelH& l = P.levels[i];
    put(b.lv[i].grp, l.grp.data(), sizeof(SegGroupH) * l.grp.size());
    put(b.lv[i].tile_grp, l.tile_grp.data(), sizeof(int32_t) * l.tile_grp.size());
    put(b.lv[i].row_grp, l.row_grp.data(), sizeof(int32_t) * l.row_grp.size());
    put(b.lv[i].run_len, l.run_len.data(), sizeof(int32_t) * l.run_len.size());
  }
}

}  // namespace gms
