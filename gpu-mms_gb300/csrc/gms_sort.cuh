// Host orchestration of the GB300 multiway mergesort.
//
// Reference counterpart: multimergesort<T,f> (GPU-MMS src/multimergesort.hxx:56-141):
// base case, then ceil(log_K(N/M)) rounds of partition + merge ping-ponging
// between `input` and `output`.
//
// Round structure here:
//   base    tile_kernel<MODE_BASE>: every CAP-key tile sorted (CAP = NT*ITEMS);
//           also writes the block sample of its output (every B-th key).
//   round p runs of length L = CAP*K^(p-1) are merged K at a time:
//     1. the block samples of the K runs of each group are merged (recursively,
//        with the same round procedure) into F, carrying each sample's index;
//     2. splitter_kernel cuts F every G entries and turns each cut into exact
//        per-run offsets (tiles of at most (G+K)*B <= CAP keys);
//     3. tile_kernel<MODE_TILE> merges each tile in shared memory and writes
//        the block sample of the output for the next round.
//   When a whole group fits one tile (K*L <= CAP) the round is a single
//   tile_kernel<MODE_GROUP> launch, which is how the recursion ends.
// The base case runs in place or out of place so that the last round always
// lands in `output`; `input` is clobbered (as in the reference).
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "gms_host_plan.h"
#include "gms_kernels.cuh"
#include "gms_seg_plan.h"

namespace gms {

constexpr int kMaxLevels = 8;

// Kernel classes for live timing and launch counting.
enum KernelClass : int {
  KC_BASE = 0,          // tile_kernel<MODE_BASE>: base-case tile sort
  KC_MERGE = 1,         // tile_kernel<GROUP/TILE> on the data (one K-way round)
  KC_SAMPLE_MERGE = 2,  // tile_kernel<GROUP/TILE> on block samples
  KC_SPLIT = 3,         // splitter_kernel
  KC_GATHER = 4,        // gather_sample_kernel
  KC_CORANK = 5,        // corank_kernel
  KC_H2D = 6,           // host-to-device input copy of a host-fed sort (not a kernel)
  KC_D2H = 7,           // device-to-host output copy of a host-fed sort (not a kernel)
  KC_COUNT = 8
};

// Optional instrumentation.  The C-ABI library installs hooks that count
// launches and, when timing is on, bracket each launch with CUDA events on the
// launching stream.  Code that includes these headers directly (the drop-in
// template) has no hooks installed.
struct Hooks {
  void (*before)(int kc, cudaStream_t st);
  void (*after)(int kc, cudaStream_t st);
};
inline Hooks* g_hooks = nullptr;
inline void hook_before(int kc, cudaStream_t st) {
  if (g_hooks) g_hooks->before(kc, st);
}
inline void hook_after(int kc, cudaStream_t st) {
  if (g_hooks) g_hooks->after(kc, st);
}

// Programmatic dependent launch of the engine's kernels (process-wide switch,
// on by default; the C ABI's gms_set_pdl sets it).
inline std::atomic<int>& pdl_enabled() {
  static std::atomic<int> on{1};
  return on;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Tunables of one sort (the autotuner picks these; defaults below).
struct Tune {
  int k = 32;         // fan-in per round (<= 32)
  int sample_b = 32;  // block size of the forecast sample
  int bulk_copy = 1;  // tile staging: 1 cp.async.bulk by one warp (3: same, persistent CTAs overlapping the
                      // next tile's staging with the store); 2 cp.async by every warp; 0 plain loads
  int split = 0;      // tile boundaries: 0 the block sample brackets each run's co-rank to one block, then a
                      // search inside it; 1 a binary search over the whole run (findPartitions-style)
  int base = 0;       // base case of keys-only integer sorts: 0 register network + warp-shuffle merges (8192-key
                      // tiles for 32-bit keys); 1 register network per thread + shared-memory merge levels
                      // (the engine's NT x ITEMS tile); other engines always use the latter
};

// Scratch layout, computed by a dry run of the same recursion as the real run.
struct WsLayout {
  int64_t s1 = 0;                      // data-level sample (two buffers)
  int64_t s[kMaxLevels] = {0};         // gathered samples, level >= 2
  int64_t f[kMaxLevels] = {0};         // merged samples (keys + index), level >= 1
  int64_t rows[kMaxLevels] = {0};      // tile boundary rows, level >= 0
  int depth = 0;
  bool ok = true;                      // false: the recursion would exceed kMaxLevels
};

template <class KeyT>
struct WsPtrs {
  int* err = nullptr;  // device status word (first 256 bytes of the scratch)
  KeyT* s1[2] = {nullptr, nullptr};
  KeyT* s[kMaxLevels] = {nullptr};
  KeyT* fk[kMaxLevels] = {nullptr};
  uint32_t* fi[kMaxLevels] = {nullptr};
  int64_t* desc[kMaxLevels] = {nullptr};
  int64_t* doff[kMaxLevels] = {nullptr};
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class KeyT>
size_t ws_bytes_for(const WsLayout& l, int k) {
  size_t b = 256;  // status word
  b += 2 * align_up(sizeof(KeyT) * (size_t)l.s1, 256);
  for (int i = 0; i < kMaxLevels; ++i) {
    b += align_up(sizeof(KeyT) * (size_t)l.s[i], 256);
    b += align_up(sizeof(KeyT) * (size_t)l.f[i], 256);
    b += align_up(sizeof(uint32_t) * (size_t)l.f[i], 256);
    b += align_up(sizeof(int64_t) * (size_t)l.rows[i] * k, 256);
    b += align_up(sizeof(int64_t) * (size_t)l.rows[i], 256);
  }
  return b + 256;
}

template <class KeyT>
WsPtrs<KeyT> ws_carve(const WsLayout& l, int k, void* base) {
  WsPtrs<KeyT> p;
  char* c = (char*)align_up((size_t)base, 256);
  auto take = [&](size_t bytes) {
    char* r = c;
    c += align_up(bytes, 256);
    return r;
  };
  p.err = (int*)take(256);
  p.s1[0] = (KeyT*)take(sizeof(KeyT) * (size_t)l.s1);
  p.s1[1] = (KeyT*)take(sizeof(KeyT) * (size_t)l.s1);
  for (int i = 0; i < kMaxLevels; ++i) {
    p.s[i] = (KeyT*)take(sizeof(KeyT) * (size_t)l.s[i]);
    p.fk[i] = (KeyT*)take(sizeof(KeyT) * (size_t)l.f[i]);
    p.fi[i] = (uint32_t*)take(sizeof(uint32_t) * (size_t)l.f[i]);
    p.desc[i] = (int64_t*)take(sizeof(int64_t) * (size_t)l.rows[i] * k);
    p.doff[i] = (int64_t*)take(sizeof(int64_t) * (size_t)l.rows[i]);
  }
  return p;
}

// Resident CTAs per SM x SM count for a persistent kernel (cached per kernel).
inline int persistent_grid(const void* kern, int threads, size_t smem, cudaError_t* err) {
  static std::mutex mu;
  static const void* keys[64];
  static int vals[64];
  static int nk = 0;
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess) return 0;
  std::lock_guard<std::mutex> g(mu);
  for (int i = 0; i < nk; ++i) {
    if (keys[i] == kern) return vals[i];
  }
  int sms = 0, per = 0;
  *err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (*err != cudaSuccess) return 0;
  *err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem);
  if (*err != cudaSuccess) return 0;
  if (per < 1) per = 1;
  const int v = sms * per;
  if (nk < 64) {
    keys[nk] = kern;
    vals[nk] = v;
    ++nk;
  }
  return v;
}

// Per-kernel, per-device opt-in to large dynamic shared memory.
// CTAs of `kern` that fit the device at once (occupancy x SMs), cached.
inline cudaError_t resident_ctas(const void* kern, int threads, size_t smem, int* out) {
  static std::mutex mu;
  static const void* seen_k[64];
  static int seen_d[64], seen_v[64];
  static int nseen = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> g(mu);
    for (int i = 0; i < nseen; ++i) {
      if (seen_k[i] == kern && seen_d[i] == dev) {
        *out = seen_v[i];
        return cudaSuccess;
      }
    }
  }
  int per_sm = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int v = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  std::lock_guard<std::mutex> g(mu);
  if (nseen < 64) {
    seen_k[nseen] = kern;
    seen_d[nseen] = dev;
    seen_v[nseen] = v;
    ++nseen;
  }
  *out = v;
  return cudaSuccess;
}

inline cudaError_t ensure_smem(const void* kern, size_t bytes) {
  static std::mutex mu;
  static const void* seen_k[256];
  static int seen_d[256];
  static int nseen = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  for (int i = 0; i < nseen; ++i) {
    if (seen_k[i] == kern && seen_d[i] == dev) return cudaSuccess;
  }
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  // largest shared-memory carveout, so several tile CTAs fit an SM
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  if (nseen < 256) {
    seen_k[nseen] = kern;
    seen_d[nseen] = dev;
    ++nseen;
  }
  return cudaSuccess;
}

// The engine for one (key, payload, comparator, codec) combination.
//   K      stored key type (unsigned for built-in dtypes)
//   V      payload type, or NoVal
//   Cmp    strict weak order on K
//   Codec  user bits <-> K
//   STABLE stable base case (key/value sorts, user comparators)
// Host-fed base case: before the base case sorts the tiles of chunk c it makes
// the stream wait for ready[c] (that chunk's input copy), so copies of later
// chunks overlap the sorting of earlier ones.  Chunk c covers base tiles
// [start[c], start[c + 1]); start holds chunks + 1 ascending offsets from 0.
//
// With `side` set (two streams) and `alt_ws` (a second scratch of the same
// layout), chunk c runs on side[c % 2] with the level buffers of its own
// scratch (the first for even chunks, alt_ws for odd ones; the data-level
// samples and the status word are shared, each chunk writing its own part),
// so the small sample merges and splitters of one chunk overlap the base case
// and merges of the next.  The side streams start after `fork` (recorded on
// the sort stream) and the sort stream waits for `join` on both before the
// rounds that span chunks.
struct BaseGate {
  int chunks = 0;
  const int64_t* start = nullptr;
  const cudaEvent_t* ready = nullptr;
  bool early_rounds = true;  // also run the merge rounds whose groups fit a chunk, chunk by chunk
  const cudaStream_t* side = nullptr;
  cudaEvent_t fork = nullptr;
  const cudaEvent_t* join = nullptr;
  void* alt_ws = nullptr;
};

// Last round in parts: the tile merge of a single-group round is launched in
// `parts` pieces of consecutive tiles, and after each piece `after(ctx, safe,
// stream)` is called with a count of leading output keys that are final once
// the piece has run.  Tiles of one group write consecutive output ranges in
// tile order, and tile T starts at or after (T*G - K)*B keys (each run has at
// most one partial sample block ahead of boundary T), so after tiles [0, T)
// at least that prefix is final.
// With `ramp` set the first two pieces hold about 1/32 and 1/16 of the tiles
// and the rest is split evenly, so the first final prefix is ready early
// (host_split_ends in gms_host_plan.h).
struct RoundSplit {
  int parts = 0;
  bool ramp = false;
  void (*after)(void* ctx, int64_t safe, cudaStream_t st) = nullptr;
  void* ctx = nullptr;
};

// Device view of one round of a segmented plan (gms_seg_plan.h): its listed
// groups and maps, and the round of its sample merges.
struct SegLevelDev {
  int64_t n = 0, L = 0, runs = 0, groups = 0, tiles = 0, rows = 0;
  bool whole = false;
  const GroupDesc* grp = nullptr;
  const int32_t* tile_grp = nullptr;
  const int32_t* row_grp = nullptr;
  const int32_t* run_len = nullptr;
  const SegLevelDev* sample = nullptr;
};
struct SegDev {
  const GroupDesc* base = nullptr;
  int64_t base_tiles = 0;
  std::vector<SegLevelDev> levels;
  std::vector<int> rounds;  // level of data rounds 1 .. R
};

// Binds a plan's levels to its arrays uploaded at `blob` (seg_blob_layout).
inline void seg_bind(const SegPlanH& P, const SegBlob& b, const void* blob, SegDev* D) {
  const unsigned char* c = static_cast<const unsigned char*>(blob);
  D->base = reinterpret_cast<const GroupDesc*>(c + b.base);
  D->base_tiles = (int64_t)P.base.size();
  D->levels.assign(P.levels.size(), SegLevelDev{});
  for (size_t i = 0; i < P.levels.size(); ++i) {
    const SegLevelH& l = P.levels[i];
    SegLevelDev& d = D->levels[i];
    d.n = l.n;
    d.L = l.L;
    d.runs = l.runs;
    d.groups = (int64_t)l.grp.size() - 1;
    d.tiles = (int64_t)l.tile_grp.size();
    d.rows = (int64_t)l.row_grp.size();
    d.whole = l.whole;
    d.grp = reinterpret_cast<const GroupDesc*>(c + b.lv[i].grp);
    d.tile_grp = reinterpret_cast<const int32_t*>(c + b.lv[i].tile_grp);
    d.row_grp = reinterpret_cast<const int32_t*>(c + b.lv[i].row_grp);
    d.run_len = reinterpret_cast<const int32_t*>(c + b.lv[i].run_len);
  }
  for (size_t i = 0; i < P.levels.size(); ++i) {
    if (P.levels[i].sample >= 0) D->levels[i].sample = &D->levels[(size_t)P.levels[i].sample];
  }
  D->rounds = P.rounds;
}

// Scratch layout of a segmented plan (same parts as a plain sort's).
inline WsLayout seg_ws_layout(const SegPlanH& P) {
  WsLayout l;
  l.s1 = P.s1;
  for (int i = 0; i < kMaxLevels && i < 8; ++i) {
    l.s[i] = P.s[i];
    l.f[i] = P.f[i];
    l.rows[i] = P.rows[i];
  }
  l.depth = P.depth;
  l.ok = P.ok;
  return l;
}

// Geometry of the merge kernels of one payload type: NT threads x ITEMS keys,
// NS merge streams per thread.  CAP bounds a group merged by one CTA
// (tile_kernel), CAPW a forecast tile (merge_tiles_kernel, window-aligned).
template <int NT_, int ITEMS_, int NS_ = 2>
struct MergeGeo {
  static constexpr int NT = NT_;
  static constexpr int ITEMS = ITEMS_;
  static constexpr int NS = NS_;
  static constexpr int CAP = NT * ITEMS;
  static constexpr int CAPW = WindowCap<NT, ITEMS>::value;
};

// Geometry of the warp-shuffle base case: NT threads x KPL keys per lane
// (tile NT*KPL), shared-memory merge levels with ITEMS outputs per thread.
template <int NT_, int KPL_, int ITEMS_, int NS_ = 2>
struct WarpBaseGeo {
  static constexpr int NT = NT_;
  static constexpr int KPL = KPL_;
  static constexpr int ITEMS = ITEMS_;
  static constexpr int NS = NS_;  // merge streams per window in the shared-memory levels
};
// 32-bit keys: 8192-key tiles; 64-bit keys: 4096-key tiles (256 threads keep
// three CTAs per SM within the register file and shared memory).  Windows of
// 65 keys in the shared-memory levels of 32-bit tiles (fewer merge-path
// searches per key: -3% base-case time against 33).
template <class KeyT>
using DefaultWarpBase = std::conditional_t<sizeof(KeyT) == 4, WarpBaseGeo<256, 32, 65>, WarpBaseGeo<256, 16, 33>>;

// MG: merge geometry of the data rounds (payload V); IG: of the rounds that
// carry a uint32 index payload (merging a block sample with its positions);
// WB: warp-shuffle base case (keys-only 4/8-byte integer keys).
template <class KeyT, class V, class Cmp, class Codec, bool STABLE, int NT, int ITEMS, class MG = MergeGeo<NT, ITEMS>,
          class IG = MG, class WB = DefaultWarpBase<KeyT>>
struct Engine {
  using IdxT = uint32_t;
  // geometry of a round whose payload is VV
  template <class VV>
  using Geo = std::conditional_t<std::is_same<VV, V>::value, MG, IG>;
  // base-case tile (NT threads x ITEMS keys)
  static constexpr int CAP = NT * ITEMS;
  // smallest forecast tile capacity over both geometries (bounds the tuning)
  static constexpr int CAPW = MG::CAPW < IG::CAPW ? MG::CAPW : IG::CAPW;
  // Keys-only sorts of 4- and 8-byte integer keys use the warp-shuffle base
  // case (geometry WB).
  static constexpr bool kWarpBase =
      !STABLE && !HasVal<V>::value && std::is_integral<KeyT>::value && (sizeof(KeyT) == 4 || sizeof(KeyT) == 8);
  static constexpr int kNTB = WB::NT;
  static constexpr int kKPL = WB::KPL;
  static constexpr int kITB = WB::ITEMS;
  static constexpr int BASE_TILE = kWarpBase ? kNTB * kKPL : CAP;

  // ---------------- geometry ----------------
  // the base case a tuning selects, and its tile
  static bool warp_base(const Tune& t) { return kWarpBase && t.base == 0; }
  static int64_t base_tile(const Tune& t) { return warp_base(t) ? (int64_t)BASE_TILE : (int64_t)CAP; }
  static int passes_for(int64_t n, const Tune& t) {
    int p = 0;
    for (int64_t L = base_tile(t); L < n; L *= t.k) ++p;
    return p;
  }

  // Walks the recursion of one merge round (payload VV) and records scratch
  // sizes.
  template <class VV = V>
  static void plan_round(WsLayout& l, int level, int64_t n, int64_t L, const Tune& t, bool gather0 = false) {
    const int k = t.k;
    if ((int64_t)k * L <= Geo<VV>::CAP) return;  // GROUP mode, no scratch
    if (level + 1 >= kMaxLevels) {
      l.ok = false;  // sample recursion too deep for this tuning
      return;
    }
    const int sb = t.sample_b;
    const int64_t G = Geo<VV>::CAPW / sb - k;
    const int64_t runs = ceil_div(n, L);
    const int64_t Ls = ceil_div(L, sb);
    const int64_t ns = (runs - 1) * Ls + ceil_div(n - (runs - 1) * L, sb);
    const int64_t groups = ceil_div(n, L * k);
    const int64_t tiles_full = ceil_div((int64_t)k * Ls, G);
    const int64_t rows = groups * (tiles_full + 1);
    l.rows[level] = std::max(l.rows[level], rows);
    l.f[level + 1] = std::max(l.f[level + 1], ns);
    if (level == 0 && !gather0) {
      l.s1 = std::max(l.s1, ns);
    } else {
      l.s[level + 1] = std::max(l.s[level + 1], ns);
    }
    l.depth = std::max(l.depth, level + 1);
    plan_round<IdxT>(l, level + 1, ns, Ls, t);
  }

  static WsLayout plan(int64_t n, const Tune& t) {
    WsLayout l;
    int64_t L = base_tile(t);
    while (L < n) {
      plan_round<V>(l, 0, n, L, t);
      L *= t.k;
    }
    return l;
  }

  template <class VV = V>
  static WsLayout plan_merge_level(int64_t n, int64_t L, const Tune& t) {
    WsLayout l;
    plan_round<VV>(l, 0, n, L, t, true);
    return l;
  }

  // ---------------- launches ----------------
  // Every engine kernel goes out with programmatic stream serialization while
  // pdl_enabled() (its launch is set up while the previous kernel runs; the
  // kernel waits in pdl_wait() for that kernel's results).
  template <class... KArgs, class... Args>
  static cudaError_t launch_kernel(void (*kern)(KArgs...), int64_t grid, int block, size_t smem, cudaStream_t st,
                                   Args... args) {
    if (grid <= 0 || grid > 0x7fffffff) return cudaErrorInvalidConfiguration;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled().load(std::memory_order_relaxed) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
  }

  template <int MODE, class VV>
  static cudaError_t launch_tile(const TileArgs<KeyT, VV>& a, int64_t grid, cudaStream_t st, int level = 0) {
    if (grid <= 0) return cudaSuccess;
    constexpr bool kStable = (MODE == MODE_BASE) ? STABLE : false;
    constexpr int kNT = (MODE == MODE_BASE) ? NT : Geo<VV>::NT;
    constexpr int kIT = (MODE == MODE_BASE) ? ITEMS : Geo<VV>::ITEMS;
    auto kern = tile_kernel<KeyT, VV, Cmp, Codec, MODE, kStable, kNT, kIT>;
    const size_t smem = TileSmemLayout<KeyT, VV, kNT * kIT>::bytes;
    cudaError_t e = ensure_smem((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    if (grid > 0x7fffffff) return cudaErrorInvalidConfiguration;
    const int kc = (MODE == MODE_BASE) ? KC_BASE : (level == 0 ? KC_MERGE : KC_SAMPLE_MERGE);
    hook_before(kc, st);
    e = launch_kernel(kern, grid, kNT, smem, st, a);
    hook_after(kc, st);
    return e;
  }

  // Warp-shuffle base case (keys-only 4/8-byte keys).
  static cudaError_t launch_base_warp(const TileArgs<KeyT, V>& a, int64_t grid, cudaStream_t st) {
    if constexpr (kWarpBase) {
      if (grid <= 0) return cudaSuccess;
      if (grid > 0x7fffffff) return cudaErrorInvalidConfiguration;
      auto kern = base_warp_kernel<KeyT, Cmp, Codec, kNTB, kKPL, kITB, WB::NS>;
      const size_t smem = BaseWarpSmem<KeyT, kNTB, kKPL, kITB, RunPad<KeyT, NoVal, Cmp, kITB, WB::NS>::gap>::bytes;
      cudaError_t e = ensure_smem((const void*)kern, smem);
      if (e != cudaSuccess) return e;
      hook_before(KC_BASE, st);
      e = launch_kernel(kern, grid, kNTB, smem, st, a);
      hook_after(KC_BASE, st);
      return e;
    } else {
      (void)a;
      (void)grid;
      (void)st;
      return cudaErrorNotSupported;
    }
  }

  // Bulk-copy merge of the forecast tiles of one round (one CTA per tile).
  template <class VV>
  // Launches blocks for tiles [a.tile_base, a.tile_base + grid) of a round
  // with `total_tiles` tiles (grid defaults to all of them).
  static cudaError_t launch_merge_tiles(const TileArgs<KeyT, VV>& a, int64_t total_tiles, cudaStream_t st,
                                        int level, int copy_mode, int64_t grid = -1) {
    if (grid < 0) grid = total_tiles - a.tile_base;
    if (grid <= 0) return cudaSuccess;
    if (grid > 0x7fffffff) return cudaErrorInvalidConfiguration;
    using GG = Geo<VV>;
    const bool persist = copy_mode == 3;
    auto kern = copy_mode == 2 ? merge_tiles_kernel<KeyT, VV, Cmp, Codec, GG::NT, GG::ITEMS, GG::NS, 2>
                : persist      ? merge_tiles_kernel<KeyT, VV, Cmp, Codec, GG::NT, GG::ITEMS, GG::NS, 1, true>
                               : merge_tiles_kernel<KeyT, VV, Cmp, Codec, GG::NT, GG::ITEMS, GG::NS, 1>;
    const size_t smem = persist ? MergeLayoutOf<KeyT, VV, Cmp, GG::NT, GG::ITEMS, GG::NS, true>::bytes
                                : MergeLayoutOf<KeyT, VV, Cmp, GG::NT, GG::ITEMS, GG::NS, false>::bytes;
    cudaError_t e = ensure_smem((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    if (persist) {
      // one wave of resident CTAs; each loops over its share of the tiles
      int slots = 0;
      e = resident_ctas((const void*)kern, GG::NT, smem, &slots);
      if (e != cudaSuccess) return e;
      grid = std::min<int64_t>(grid, slots);
    }
    const int kc = level == 0 ? KC_MERGE : KC_SAMPLE_MERGE;
    hook_before(kc, st);
    e = launch_kernel(kern, grid, GG::NT, smem, st, a, total_tiles);
    hook_after(kc, st);
    return e;
  }

  // One K-way round over runs of length L.  `sample_in` is the block sample of
  // `in` (null: gather it here); `sample_out` receives the block sample of the
  // output runs (null: not needed).
  // Segmented rounds (sl set): the groups are listed by the plan level `sl`,
  // groups flagged GRP_ALT read in2/vin2 and write out2/vout2, and the round
  // never uses the plain-load tile path (staging mode 0 runs as mode 1).
  template <class VV>
  static cudaError_t round(const WsPtrs<KeyT>& w, int level, const KeyT* in, const VV* vin, KeyT* out, VV* vout, int64_t n,
                           int64_t L, const Tune& t, const KeyT* sample_in, KeyT* sample_out, int enc, int dec,
                           int gen_index, cudaStream_t st, const RoundSplit* split = nullptr,
                           const SegLevelDev* sl = nullptr, const KeyT* in2 = nullptr, KeyT* out2 = nullptr,
                           const VV* vin2 = nullptr, VV* vout2 = nullptr) {
    const int k = t.k;
    const int sb = t.sample_b;
    TileArgs<KeyT, VV> a{};
    if (sl) {
      a.grp = sl->grp;
      a.tile_grp = sl->tile_grp;
      a.in2 = in2;
      a.out2 = out2;
      a.vin2 = vin2;
      a.vout2 = vout2;
    }
    a.in = in;
    a.out = out;
    a.vin = vin;
    a.vout = vout;
    a.n = n;
    a.L = L;
    a.k = k;
    a.enc_on_load = enc;
    a.dec_on_store = dec;
    a.gen_index = gen_index;
    a.err = w.err;
    a.sample_out = sample_out;
    a.sample_b = sb;
    a.out_run_len = L * k;
    a.sample_run_len = ceil_div(L * k, sb);
    const int64_t groups = sl ? sl->groups : ceil_div(n, L * k);
    a.groups = groups;
    if ((int64_t)k * L <= Geo<VV>::CAP) {
      return launch_tile<MODE_GROUP>(a, groups, st, level);
    }
    if (level + 1 >= kMaxLevels) return cudaErrorInvalidValue;
    const int64_t G = Geo<VV>::CAPW / sb - k;
    const int64_t runs = sl ? sl->runs : ceil_div(n, L);
    const int64_t Ls = ceil_div(L, sb);
    // listed groups keep every run's block sample Ls apart (gaps after short runs)
    const int64_t ns = sl ? runs * Ls : (runs - 1) * Ls + ceil_div(n - (runs - 1) * L, sb);
    cudaError_t e;
    const KeyT* S = sample_in;
    if (!S) {
      KeyT* g = w.s[level + 1];
      const int64_t slots = runs * Ls;
      hook_before(KC_GATHER, st);
      e = launch_kernel(gather_sample_kernel<KeyT, Codec>, ceil_div(slots, 256), 256, 0, st, in, g, n, L, Ls, sb,
                        slots, enc, sl ? sl->run_len : nullptr);
      hook_after(KC_GATHER, st);
      if (e != cudaSuccess) return e;
      S = g;
    }
    // 1. merge the block samples of each group, keeping each sample's index
    e = round<IdxT>(w, level + 1, S, nullptr, w.fk[level + 1], w.fi[level + 1], ns, Ls, t, nullptr, nullptr, 0, 0, 1,
                    st, nullptr, sl ? sl->sample : nullptr);
    if (e != cudaSuccess) return e;
    // 2. tile boundaries
    const int64_t tiles_full = ceil_div((int64_t)k * Ls, G);
    const int64_t last_ns = ns - (groups - 1) * (int64_t)k * Ls;
    const int64_t tiles_last = ceil_div(last_ns, G);
    const int64_t rows = sl ? sl->rows : groups * (tiles_full + 1);
    {
      const int64_t threads = rows * 32;
      hook_before(KC_SPLIT, st);
      e = launch_kernel(splitter_kernel<KeyT, Cmp, Codec>, ceil_div(threads, 256), 256, 0, st, in, S,
                        (const KeyT*)w.fk[level + 1], (const uint32_t*)w.fi[level + 1], n, L, k, Ls, sb, G, tiles_full,
                        tiles_last, groups, w.desc[level], w.doff[level], enc, sl ? sl->grp : nullptr,
                        sl ? sl->row_grp : nullptr, in2, t.split);
      hook_after(KC_SPLIT, st);
      if (e != cudaSuccess) return e;
    }
    // 3. merge the tiles
    a.desc = w.desc[level];
    a.doff = w.doff[level];
    a.tiles_full = tiles_full;
    a.tiles_last = tiles_last;
    if (sl) return launch_merge_tiles(a, sl->tiles, st, level, t.bulk_copy ? t.bulk_copy : 1);
    if (t.bulk_copy && split && split->parts > 1 && groups == 1 && tiles_last > 1) {
      int64_t ends[kMaxParts];
      const int np = host_split_ends(tiles_last, split->parts, split->ramp, ends);
      int64_t t0 = 0;
      for (int i = 0; i < np; ++i) {
        const int64_t t1 = ends[i];
        if (t1 <= t0) continue;
        TileArgs<KeyT, VV> b = a;
        b.tile_base = t0;
        e = launch_merge_tiles(b, t1, st, level, t.bulk_copy, t1 - t0);
        if (e != cudaSuccess) return e;
        const int64_t safe = (t1 == tiles_last) ? n : std::max<int64_t>(0, (t1 * G - k) * (int64_t)sb);
        split->after(split->ctx, std::min(safe, n), st);
        t0 = t1;
      }
      return cudaSuccess;
    }
    if (t.bulk_copy) return launch_merge_tiles(a, groups * tiles_full, st, level, t.bulk_copy);
    return launch_tile<MODE_TILE>(a, groups * tiles_full, st, level);
  }

  // Full sort.  Result in `out` (keys) / `vout` (payload); `in`/`vin` are
  // clobbered.  The base case runs in place when the round count is odd, so
  // the last round lands in `out`.
  static cudaError_t sort(const WsPtrs<KeyT>& w, KeyT* in, V* vin, KeyT* out, V* vout, int64_t n, const Tune& t,
                          cudaStream_t st, const BaseGate* gate = nullptr, const RoundSplit* split = nullptr) {
    const bool odd = passes_for(n, t) % 2 == 1;
    return sort_to(w, in, vin, odd ? in : out, odd ? vin : vout, odd ? out : in, odd ? vout : vin, out, vout, n, t, st,
                   gate, split);
  }

  // Full sort with explicit buffers: the base case reads `src` and writes
  // `d0` (or `dst` when no merge round follows), rounds ping-pong between `d0`
  // and `d1`, and the last round writes `dst`.  `src` may equal `d0`; `dst`
  // must differ from the last round's input (d0 when the round count is odd,
  // d1 when it is even) and may be any memory the kernels can store to,
  // mapped pinned host memory included.
  static cudaError_t sort_to(const WsPtrs<KeyT>& w, const KeyT* src, const V* vsrc, KeyT* d0, V* vd0, KeyT* d1, V* vd1,
                             KeyT* dst, V* vdst, int64_t n, const Tune& t, cudaStream_t st,
                             const BaseGate* gate = nullptr, const RoundSplit* split = nullptr) {
    if (n <= 0) return cudaSuccess;
    const int P = passes_for(n, t);
    const int64_t bt = base_tile(t);
    KeyT* buf[2] = {d0, d1};
    V* vbuf[2] = {vd0, vd1};
    int rounds_done = 0;  // rounds already run chunk by chunk
    {
      TileArgs<KeyT, V> a{};
      a.in = src;
      a.out = P > 0 ? d0 : dst;
      a.vin = vsrc;
      a.vout = P > 0 ? vd0 : vdst;
      a.n = n;
      a.L = bt;
      a.k = 1;
      a.enc_on_load = 1;
      a.dec_on_store = (P == 0) ? 1 : 0;
      a.gen_index = 0;
      a.err = w.err;
      a.sample_b = t.sample_b;
      a.out_run_len = bt;
      a.sample_run_len = ceil_div(bt, t.sample_b);
      a.sample_out = (P > 0) ? w.s1[0] : nullptr;
      cudaError_t e = cudaSuccess;
      if (warp_base(t)) {
        const int64_t tiles = ceil_div(n, BASE_TILE);
        if (!gate) {
          e = launch_base_warp(a, tiles, st);
        } else {
          // Host-fed: each chunk is sorted as far as it can be on its own --
          // the base case and every round but the last whose groups fit whole
          // inside a chunk -- as soon as its copy lands.
          // rounds whose groups start on every interior chunk boundary
          int pc = 0;
          for (int64_t gk = t.k; gate->early_rounds && pc < P - 1; gk *= t.k) {
            bool whole = true;
            for (int c = 1; c < gate->chunks && whole; ++c)
              whole = gate->start[c] >= tiles || gate->start[c] % gk == 0;
            if (!whole) break;
            ++pc;
          }
          const bool two = gate->side && gate->alt_ws && gate->fork && gate->join;
          WsPtrs<KeyT> wa = w;
          if (two) {
            wa = ws_carve<KeyT>(plan(n, t), t.k, gate->alt_ws);
            wa.err = w.err;
            wa.s1[0] = w.s1[0];
            wa.s1[1] = w.s1[1];
            e = cudaEventRecord(gate->fork, st);
            for (int j = 0; j < 2 && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(gate->side[j], gate->fork, 0);
          }
          for (int c = 0; c < gate->chunks && e == cudaSuccess; ++c) {
            const int64_t t0 = gate->start[c];
            if (t0 >= tiles) break;
            const int64_t t1 = std::min(tiles, gate->start[c + 1]);
            const cudaStream_t cs = two ? gate->side[c & 1] : st;
            const WsPtrs<KeyT>& wc = (two && (c & 1)) ? wa : w;
            e = cudaStreamWaitEvent(cs, gate->ready[c], 0);
            if (e != cudaSuccess) break;
            TileArgs<KeyT, V> b = a;
            const int64_t off = t0 * BASE_TILE;
            const int64_t nc = std::min(n, t1 * BASE_TILE) - off;
            b.in = a.in + off;
            b.out = a.out + off;
            b.n = nc;
            b.sample_out = a.sample_out ? a.sample_out + t0 * a.sample_run_len : nullptr;
            e = launch_base_warp(b, t1 - t0, cs);
            int cc = 0, sb = 0;
            int64_t L = BASE_TILE;
            for (int p = 0; p < pc && e == cudaSuccess; ++p) {
              const int64_t lk = L * t.k;
              const KeyT* sin = w.s1[sb] + (off / L) * ceil_div(L, t.sample_b);
              KeyT* sout = w.s1[sb ^ 1] + (off / lk) * ceil_div(lk, t.sample_b);
              e = round<V>(wc, 0, buf[cc] + off, vbuf[cc] ? vbuf[cc] + off : nullptr, buf[cc ^ 1] + off,
                           vbuf[cc ^ 1] ? vbuf[cc ^ 1] + off : nullptr, nc, L, t, sin, sout, 0, 0, 0, cs);
              cc ^= 1;
              sb ^= 1;
              L = lk;
            }
          }
          if (two) {
            for (int j = 0; j < 2; ++j) {
              const cudaError_t ej = cudaEventRecord(gate->join[j], gate->side[j]);
              const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(st, gate->join[j], 0) : ej;
              if (e == cudaSuccess) e = ew;
            }
          }
          rounds_done = pc;
        }
      } else {
        for (int c = 0; gate && c < gate->chunks && e == cudaSuccess; ++c) e = cudaStreamWaitEvent(st, gate->ready[c], 0);
        if (e == cudaSuccess) e = launch_tile<MODE_BASE>(a, ceil_div(n, CAP), st);
      }
      if (e != cudaSuccess) return e;
    }
    int cur = rounds_done & 1;
    int sbuf = rounds_done & 1;
    int64_t L = bt;
    for (int p = 0; p < rounds_done; ++p) L *= t.k;
    for (int p = rounds_done; p < P; ++p) {
      const bool last = (p == P - 1);
      KeyT* sout = last ? nullptr : w.s1[sbuf ^ 1];
      KeyT* o = last ? dst : buf[cur ^ 1];
      V* vo = last ? vdst : vbuf[cur ^ 1];
      cudaError_t e = round<V>(w, 0, buf[cur], vbuf[cur], o, vo, n, L, t, w.s1[sbuf], sout, 0, last ? 1 : 0, 0, st,
                               last ? split : nullptr);
      if (e != cudaSuccess) return e;
      cur ^= 1;
      sbuf ^= 1;
      L *= t.k;
    }
    return cudaSuccess;
  }

  // ---------------- segmented sorts ----------------
  static SegGeom seg_geom(const Tune& t) {
    SegGeom g;
    g.base_tile = base_tile(t);
    g.cap_data = Geo<V>::CAP;
    g.capw_data = Geo<V>::CAPW;
    g.cap_idx = Geo<IdxT>::CAP;
    g.capw_idx = Geo<IdxT>::CAPW;
    g.k = t.k;
    g.sample_b = t.sample_b;
    g.max_levels = kMaxLevels;
    return g;
  }

  // Sorts every segment of a plan bound as D: `src` (n keys, with payload
  // `vsrc`) is read only, `tmp` is scratch of n keys (+ payload), the sorted
  // segments land in `dst`.  One base-case launch over every segment's tiles,
  // then one launch sequence per round over the groups of the segments that
  // still need it; each segment's last round (or its base case) writes `dst`.
  static cudaError_t seg_sort(const WsPtrs<KeyT>& w, const SegDev& D, const KeyT* src, const V* vsrc, KeyT* tmp,
                              V* vtmp, KeyT* dst, V* vdst, int64_t n, const Tune& t0, cudaStream_t st) {
    if (n <= 0 || D.base_tiles == 0) return cudaSuccess;
    Tune t = t0;
    if (t.bulk_copy == 0) t.bulk_copy = 1;
    const int R = (int)D.rounds.size();
    TileArgs<KeyT, V> a{};
    a.in = src;
    a.out = tmp;
    a.vin = vsrc;
    a.vout = vtmp;
    a.in2 = src;
    a.out2 = dst;
    a.vin2 = vsrc;
    a.vout2 = vdst;
    const int64_t bt = base_tile(t);
    a.n = n;
    a.L = bt;
    a.k = 1;
    a.enc_on_load = 1;
    a.dec_on_store = 0;
    a.err = w.err;
    a.grp = D.base;
    a.sample_b = t.sample_b;
    a.out_run_len = bt;
    a.sample_run_len = ceil_div(bt, t.sample_b);
    a.sample_out = R > 0 ? w.s1[0] : nullptr;
    cudaError_t e = warp_base(t) ? launch_base_warp(a, D.base_tiles, st) : launch_tile<MODE_BASE>(a, D.base_tiles, st);
    if (e != cudaSuccess) return e;
    int64_t L = bt;
    for (int p = 0; p < R; ++p, L *= t.k) {
      const SegLevelDev* sl = &D.levels[(size_t)D.rounds[(size_t)p]];
      KeyT* sout = (p + 1 < R) ? w.s1[(p + 1) & 1] : nullptr;
      e = round<V>(w, 0, tmp, vtmp, dst, vdst, n, L, t, w.s1[p & 1], sout, 0, 0, 0, st, nullptr, sl, dst, tmp, vdst,
                   vtmp);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }

  // One merge round on caller data (the multimergeLevel contract).
  static cudaError_t merge_level(const WsPtrs<KeyT>& w, const KeyT* in, KeyT* out, int64_t n, int64_t L, const Tune& t,
                                 cudaStream_t st) {
    return round<V>(w, 0, in, nullptr, out, nullptr, n, L, t, nullptr, nullptr, 1, 1, 0, st);
  }

  // Base case only: every `tile`-key tile sorted (the squareSort contract).
  static cudaError_t tile_sort(KeyT* data, int64_t n, int64_t tile, cudaStream_t st) {
    TileArgs<KeyT, V> a{};
    a.in = data;
    a.out = data;
    a.n = n;
    a.L = tile;
    a.k = 1;
    a.enc_on_load = 1;
    a.dec_on_store = 1;
    a.sample_b = 1;
    return launch_tile<MODE_BASE>(a, ceil_div(n, tile), st);
  }
};

}  // namespace gms
