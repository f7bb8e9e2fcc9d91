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
#include <cstdint>
#include <cstring>
#include <mutex>

#include "gms_kernels.cuh"

namespace gms {

constexpr int kMaxLevels = 8;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Tunables of one sort (the autotuner picks these; defaults below).
struct Tune {
  int k = 32;         // fan-in per round (<= 32)
  int sample_b = 32;  // block size of the forecast sample
};

// Scratch layout, computed by a dry run of the same recursion as the real run.
struct WsLayout {
  int64_t s1 = 0;                      // data-level sample (two buffers)
  int64_t s[kMaxLevels] = {0};         // gathered samples, level >= 2
  int64_t f[kMaxLevels] = {0};         // merged samples (keys + index), level >= 1
  int64_t rows[kMaxLevels] = {0};      // tile boundary rows, level >= 0
  int depth = 0;
};

template <class K>
struct WsPtrs {
  int* err = nullptr;  // device status word (first 256 bytes of the scratch)
  K* s1[2] = {nullptr, nullptr};
  K* s[kMaxLevels] = {nullptr};
  K* fk[kMaxLevels] = {nullptr};
  uint32_t* fi[kMaxLevels] = {nullptr};
  int64_t* desc[kMaxLevels] = {nullptr};
  int64_t* doff[kMaxLevels] = {nullptr};
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

template <class K>
size_t ws_bytes_for(const WsLayout& l, int k) {
  size_t b = 256;  // status word
  b += 2 * align_up(sizeof(K) * (size_t)l.s1, 256);
  for (int i = 0; i < kMaxLevels; ++i) {
    b += align_up(sizeof(K) * (size_t)l.s[i], 256);
    b += align_up(sizeof(K) * (size_t)l.f[i], 256);
    b += align_up(sizeof(uint32_t) * (size_t)l.f[i], 256);
    b += align_up(sizeof(int64_t) * (size_t)l.rows[i] * k, 256);
    b += align_up(sizeof(int64_t) * (size_t)l.rows[i], 256);
  }
  return b + 256;
}

template <class K>
WsPtrs<K> ws_carve(const WsLayout& l, int k, void* base) {
  WsPtrs<K> p;
  char* c = (char*)align_up((size_t)base, 256);
  auto take = [&](size_t bytes) {
    char* r = c;
    c += align_up(bytes, 256);
    return r;
  };
  p.err = (int*)take(256);
  p.s1[0] = (K*)take(sizeof(K) * (size_t)l.s1);
  p.s1[1] = (K*)take(sizeof(K) * (size_t)l.s1);
  for (int i = 0; i < kMaxLevels; ++i) {
    p.s[i] = (K*)take(sizeof(K) * (size_t)l.s[i]);
    p.fk[i] = (K*)take(sizeof(K) * (size_t)l.f[i]);
    p.fi[i] = (uint32_t*)take(sizeof(uint32_t) * (size_t)l.f[i]);
    p.desc[i] = (int64_t*)take(sizeof(int64_t) * (size_t)l.rows[i] * k);
    p.doff[i] = (int64_t*)take(sizeof(int64_t) * (size_t)l.rows[i]);
  }
  return p;
}

// Per-kernel, per-device opt-in to large dynamic shared memory.
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
template <class K, class V, class Cmp, class Codec, bool STABLE, int NT, int ITEMS>
struct Engine {
  static constexpr int CAP = NT * ITEMS;
  using IdxT = uint32_t;

  // ---------------- geometry ----------------
  static int passes_for(int64_t n, int k) {
    int p = 0;
    for (int64_t L = CAP; L < n; L *= k) ++p;
    return p;
  }

  // Walks the recursion of one merge round and records scratch sizes.
  static void plan_round(WsLayout& l, int level, int64_t n, int64_t L, const Tune& t, bool gather0 = false) {
    const int k = t.k;
    if ((int64_t)k * L <= CAP) return;  // GROUP mode, no scratch
    const int B = t.sample_b;
    const int64_t G = CAP / B - k;
    const int64_t runs = ceil_div(n, L);
    const int64_t Ls = ceil_div(L, B);
    const int64_t ns = (runs - 1) * Ls + ceil_div(n - (runs - 1) * L, B);
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
    plan_round(l, level + 1, ns, Ls, t);
  }

  static WsLayout plan(int64_t n, const Tune& t) {
    WsLayout l;
    int64_t L = CAP;
    while (L < n) {
      plan_round(l, 0, n, L, t);
      L *= t.k;
    }
    return l;
  }

  static WsLayout plan_merge_level(int64_t n, int64_t L, const Tune& t) {
    WsLayout l;
    plan_round(l, 0, n, L, t, true);
    return l;
  }

  // ---------------- launches ----------------
  template <int MODE, class VV>
  static cudaError_t launch_tile(const TileArgs<K, VV>& a, int64_t grid, cudaStream_t st) {
    if (grid <= 0) return cudaSuccess;
    constexpr bool kStable = (MODE == MODE_BASE) ? STABLE : false;
    auto kern = tile_kernel<K, VV, Cmp, Codec, MODE, kStable, NT, ITEMS>;
    const size_t smem = TileSmemLayout<K, VV, CAP>::bytes;
    cudaError_t e = ensure_smem((const void*)kern, smem);
    if (e != cudaSuccess) return e;
    if (grid > 0x7fffffff) return cudaErrorInvalidConfiguration;
    kern<<<(unsigned)grid, NT, smem, st>>>(a);
    return cudaGetLastError();
  }

  // One K-way round over runs of length L.  `sample_in` is the block sample of
  // `in` (null: gather it here); `sample_out` receives the block sample of the
  // output runs (null: not needed).
  template <class VV>
  static cudaError_t round(const WsPtrs<K>& w, int level, const K* in, const VV* vin, K* out, VV* vout, int64_t n,
                           int64_t L, const Tune& t, const K* sample_in, K* sample_out, int enc, int dec,
                           int gen_index, cudaStream_t st) {
    const int k = t.k;
    const int B = t.sample_b;
    TileArgs<K, VV> a{};
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
    a.sample_b = B;
    a.out_run_len = L * k;
    a.sample_run_len = ceil_div(L * k, B);
    const int64_t groups = ceil_div(n, L * k);
    if ((int64_t)k * L <= CAP) {
      return launch_tile<MODE_GROUP>(a, groups, st);
    }
    if (level + 1 >= kMaxLevels) return cudaErrorInvalidValue;
    const int64_t G = CAP / B - k;
    const int64_t runs = ceil_div(n, L);
    const int64_t Ls = ceil_div(L, B);
    const int64_t ns = (runs - 1) * Ls + ceil_div(n - (runs - 1) * L, B);
    cudaError_t e;
    const K* S = sample_in;
    if (!S) {
      K* g = w.s[level + 1];
      const int64_t slots = runs * Ls;
      gather_sample_kernel<K, Codec><<<(unsigned)ceil_div(slots, 256), 256, 0, st>>>(in, g, n, L, Ls, B, slots, enc);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      S = g;
    }
    // 1. merge the block samples of each group, keeping each sample's index
    e = round<IdxT>(w, level + 1, S, nullptr, w.fk[level + 1], w.fi[level + 1], ns, Ls, t, nullptr, nullptr, 0, 0, 1,
                    st);
    if (e != cudaSuccess) return e;
    // 2. tile boundaries
    const int64_t tiles_full = ceil_div((int64_t)k * Ls, G);
    const int64_t last_ns = ns - (groups - 1) * (int64_t)k * Ls;
    const int64_t tiles_last = ceil_div(last_ns, G);
    const int64_t rows = groups * (tiles_full + 1);
    {
      const int64_t threads = rows * 32;
      splitter_kernel<K, Cmp, Codec><<<(unsigned)ceil_div(threads, 256), 256, 0, st>>>(
          in, w.fk[level + 1], w.fi[level + 1], n, L, k, Ls, B, G, tiles_full, tiles_last, groups, w.desc[level],
          w.doff[level], enc);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // 3. merge the tiles
    a.desc = w.desc[level];
    a.doff = w.doff[level];
    a.tiles_full = tiles_full;
    a.tiles_last = tiles_last;
    a.groups = groups;
    return launch_tile<MODE_TILE>(a, groups * tiles_full, st);
  }

  // Full sort.  Result in `out` (keys) / `vout` (payload); `in`/`vin` are
  // clobbered.  enc/dec: apply the codec on the first load / last store.
  static cudaError_t sort(const WsPtrs<K>& w, K* in, V* vin, K* out, V* vout, int64_t n, const Tune& t,
                          cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int P = passes_for(n, t.k);
    K* buf[2] = {in, out};
    V* vbuf[2] = {vin, vout};
    // base case: P odd -> in place on `in`; P even -> `in` to `out`
    int cur = (P % 2 == 1) ? 0 : 1;
    {
      TileArgs<K, V> a{};
      a.in = in;
      a.out = buf[cur];
      a.vin = vin;
      a.vout = vbuf[cur];
      a.n = n;
      a.L = CAP;
      a.k = 1;
      a.enc_on_load = 1;
      a.dec_on_store = (P == 0) ? 1 : 0;
      a.gen_index = 0;
      a.err = w.err;
      a.sample_b = t.sample_b;
      a.out_run_len = CAP;
      a.sample_run_len = ceil_div(CAP, t.sample_b);
      a.sample_out = (P > 0) ? w.s1[0] : nullptr;
      cudaError_t e = launch_tile<MODE_BASE>(a, ceil_div(n, CAP), st);
      if (e != cudaSuccess) return e;
    }
    int sbuf = 0;
    int64_t L = CAP;
    for (int p = 0; p < P; ++p) {
      const bool last = (p == P - 1);
      K* sout = last ? nullptr : w.s1[sbuf ^ 1];
      cudaError_t e = round<V>(w, 0, buf[cur], vbuf[cur], buf[cur ^ 1], vbuf[cur ^ 1], n, L, t, w.s1[sbuf], sout, 0,
                               last ? 1 : 0, 0, st);
      if (e != cudaSuccess) return e;
      cur ^= 1;
      sbuf ^= 1;
      L *= t.k;
    }
    return cudaSuccess;
  }

  // One merge round on caller data (the multimergeLevel contract).
  static cudaError_t merge_level(const WsPtrs<K>& w, const K* in, K* out, int64_t n, int64_t L, const Tune& t,
                                 cudaStream_t st) {
    return round<V>(w, 0, in, nullptr, out, nullptr, n, L, t, nullptr, nullptr, 1, 1, 0, st);
  }

  // Base case only: every `tile`-key tile sorted (the squareSort contract).
  static cudaError_t tile_sort(K* data, int64_t n, int64_t tile, cudaStream_t st) {
    TileArgs<K, V> a{};
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
