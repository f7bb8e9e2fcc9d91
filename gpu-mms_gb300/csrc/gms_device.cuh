// Device building blocks of the GB300 multiway mergesort.
//
// Reference counterparts (GPU-MMS, paths relative to its src/):
//   cmpSwap / swap* / myMin / myMax        basecase/util.hxx:39-215
//   bitonicSort32 (register network)       basecase/sortRowMajor.hxx:96-119
//   shfl_wrapper / SHFL_XOR                basecase/sortRowMajor.hxx:36-42, params.h:40-50
//   xorMergeNodes / xorMergeGeneral        io-merge-gen.hxx:48-93, 204-236
//
// The reference merges 32-key heap nodes with warp-shuffle bitonic networks.
// Here a merge step is a merge-path split (binary search on one diagonal)
// followed by a branch-free serial merge of ITEMS keys per thread out of shared
// memory: about log2(K) comparisons per key per K-way round instead of a
// bitonic network per heap level.
#pragma once

#include <cstdint>
#include <utility>

#include <cuda_runtime.h>

namespace gms {

// ---------------------------------------------------------------------------
// Payload marker for keys-only sorts.
struct NoVal {};

template <class V>
struct HasVal {
  static constexpr bool value = true;
};
template <>
struct HasVal<NoVal> {
  static constexpr bool value = false;
};

// ---------------------------------------------------------------------------
// Codecs map a user key's bit pattern to an unsigned key whose `<` order is
// the user order, and back.  The first pass encodes on load, the last pass
// decodes on store; every pass in between compares plain unsigned integers.
template <class KeyT>
struct IdentityCodec {
  static __device__ __forceinline__ KeyT enc(KeyT x) { return x; }
  static __device__ __forceinline__ KeyT dec(KeyT x) { return x; }
};
// two's-complement order -> unsigned order
struct SignFlip32 {
  static __device__ __forceinline__ uint32_t enc(uint32_t x) { return x ^ 0x80000000u; }
  static __device__ __forceinline__ uint32_t dec(uint32_t x) { return x ^ 0x80000000u; }
};
struct SignFlip64 {
  static __device__ __forceinline__ uint64_t enc(uint64_t x) { return x ^ 0x8000000000000000ull; }
  static __device__ __forceinline__ uint64_t dec(uint64_t x) { return x ^ 0x8000000000000000ull; }
};
// IEEE-754 totalOrder over bit patterns: -NaN < -Inf < ... < -0 < +0 < ... < +Inf < +NaN
struct FloatOrder32 {
  static __device__ __forceinline__ uint32_t enc(uint32_t b) {
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
  }
  static __device__ __forceinline__ uint32_t dec(uint32_t k) {
    return (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  }
};
struct FloatOrder64 {
  static __device__ __forceinline__ uint64_t enc(uint64_t b) {
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
  }
  static __device__ __forceinline__ uint64_t dec(uint64_t k) {
    return (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  }
};

// Default strict weak order on the stored keys.
struct KeyLess {
  template <class KeyT>
  __device__ __forceinline__ bool operator()(const KeyT& a, const KeyT& b) const {
    return a < b;
  }
};

// ---------------------------------------------------------------------------
// Register sorting networks.  Indices are compile-time after unrolling, so the
// keys stay in registers (no local memory).

// Compare-exchange: afterwards a <= b.  Not stable (used where equivalent keys
// are bit-identical).
template <class KeyT, class Cmp>
__device__ __forceinline__ void cas(KeyT& a, KeyT& b, Cmp cmp) {
  const bool sw = cmp(b, a);
  const KeyT lo = sw ? b : a;
  const KeyT hi = sw ? a : b;
  a = lo;
  b = hi;
}

// Batcher odd-even merge sort for N keys, pruned from the next power of two.
// A comparator whose upper index is >= N only ever meets a virtual +inf there
// and is dropped.  The comparator list is built at compile time and expanded
// by template recursion, so every index is a constant.
struct NetTable {
  int a[1024];
  int b[1024];
  int n;
};

constexpr NetTable batcher_table(int N) {
  NetTable t{};
  t.n = 0;
  int P = 1;
  while (P < N) P *= 2;
  for (int p = 1; p < P; p *= 2) {
    for (int k = p; k >= 1; k /= 2) {
      for (int j = k % p; j + k < P; j += 2 * k) {
        for (int i = 0; i < k; ++i) {
          if (i + j + k < N && (i + j) / (2 * p) == (i + j + k) / (2 * p)) {
            t.a[t.n] = i + j;
            t.b[t.n] = i + j + k;
            ++t.n;
          }
        }
      }
    }
  }
  return t;
}

template <int N>
struct Batcher {
  static constexpr NetTable table = batcher_table(N);
};

template <int N, class KeyT, class Cmp, int... I>
__device__ __forceinline__ void network_apply(KeyT (&r)[N], Cmp cmp, std::integer_sequence<int, I...>) {
  (cas(r[Batcher<N>::table.a[I]], r[Batcher<N>::table.b[I]], cmp), ...);
}

template <int N, class KeyT, class Cmp>
__device__ __forceinline__ void network_sort(KeyT (&r)[N], Cmp cmp) {
  network_apply<N>(r, cmp, std::make_integer_sequence<int, Batcher<N>::table.n>{});
}

// Odd-even transposition sort: only adjacent keys are exchanged, and only when
// strictly out of order, so equal keys keep their order (stable).  Carries a
// payload along.
template <int N, class KeyT, class V, class Cmp>
__device__ __forceinline__ void transposition_sort(KeyT (&r)[N], V (&v)[N], Cmp cmp) {
#pragma unroll
  for (int round = 0; round < N; ++round) {
#pragma unroll
    for (int i = round & 1; i + 1 < N; i += 2) {
      const bool sw = cmp(r[i + 1], r[i]);
      const KeyT klo = sw ? r[i + 1] : r[i];
      const KeyT khi = sw ? r[i] : r[i + 1];
      r[i] = klo;
      r[i + 1] = khi;
      if constexpr (HasVal<V>::value) {
        const V vlo = sw ? v[i + 1] : v[i];
        const V vhi = sw ? v[i] : v[i + 1];
        v[i] = vlo;
        v[i + 1] = vhi;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Merge path: number of elements of `a` among the first `diag` outputs of the
// stable merge of a and b (a wins ties).  Lower-bound search whose steps are
// branch-free (selects), so lanes of a warp never diverge inside a step.
template <class KeyT, class Cmp>
__device__ __forceinline__ int merge_path(const KeyT* a, int na, const KeyT* b, int nb, int diag, Cmp cmp) {
  int lo = diag - nb > 0 ? diag - nb : 0;
  int len = (diag < na ? diag : na) - lo;
  while (len > 0) {
    const int half = len >> 1;
    const int mid = lo + half;
    const bool go = !cmp(b[diag - 1 - mid], a[mid]);
    lo = go ? mid + 1 : lo;
    len = go ? len - half - 1 : half;
  }
  return lo;
}

// Cursor of a stable two-way merge over shared memory.  A = [xa, ea),
// B = [xb, eb) (absolute indices in one buffer).  ka/kb hold the heads and
// na_/nb_ the element after each head, so the shared-memory load issued by a
// step (two past the consumed element) is only needed two steps later: the
// load latency leaves the per-step dependency chain, which is then just
// compare -> select.  step() emits the smaller head (A wins ties); no branches.
// Loads may run up to two elements past a run end, so every buffer carries
// slack elements.
template <class KeyT>
struct MergeCursor {
  int xa, ea, xb, eb;
  KeyT ka, kb, na_, nb_;

  template <class Cmp>
  __device__ __forceinline__ void init(const KeyT* sk, int a0, int a1, int b0, int b1, Cmp) {
    xa = a0;
    ea = a1;
    xb = b0;
    eb = b1;
    ka = sk[a0];
    na_ = sk[a0 + 1];
    kb = sk[b0];
    nb_ = sk[b0 + 1];
  }

  // Returns the emitted key; `src` receives its index, `took_a` its side.
  template <class Cmp>
  __device__ __forceinline__ KeyT step(const KeyT* sk, Cmp cmp, int& src, bool& took_a) {
    const bool ta = (xb >= eb) || ((xa < ea) && !cmp(kb, ka));
    const KeyT o = ta ? ka : kb;
    const int cur = ta ? xa : xb;
    const KeyT far = sk[cur + 2];
    ka = ta ? na_ : ka;
    na_ = ta ? far : na_;
    kb = ta ? kb : nb_;
    nb_ = ta ? nb_ : far;
    xa = ta ? cur + 1 : xa;
    xb = ta ? xb : cur + 1;
    src = cur;
    took_a = ta;
    return o;
  }

  __device__ __forceinline__ bool exhausted() const { return xa + xb == ea + eb; }
};

// One level of pairwise merging over runs of equal length `rl` inside a
// shared-memory tile of `cap` keys.  Thread `t` produces outputs
// [t*ITEMS, t*ITEMS + ITEMS) into registers.  ITEMS divides rl, so a thread
// never straddles two pairs.
template <int ITEMS, class KeyT, class V, class Cmp>
__device__ __forceinline__ void merge_level_regular(const KeyT* sk, const V* sv, int cap, int rl, int s,
                                                    KeyT (&ok)[ITEMS], V (&ov)[ITEMS], Cmp cmp) {
  const int ps = (s / (2 * rl)) * (2 * rl);
  const int pm = min(ps + rl, cap);
  const int pe = min(ps + 2 * rl, cap);
  const int diag = s - ps;
  const int ia = merge_path(sk + ps, pm - ps, sk + pm, pe - pm, diag, cmp);
  MergeCursor<KeyT> c;
  c.init(sk, ps + ia, pm, pm + (diag - ia), pe, cmp);
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    int src;
    bool ta;
    ok[i] = c.step(sk, cmp, src, ta);
    if constexpr (HasVal<V>::value) ov[i] = sv[src];
  }
}

// Locates the pair of level `span` that holds output position q: the largest
// pair index whose start pre[p*span] is <= q.
__device__ __forceinline__ int find_pair(const int* pre, int npairs, int span, int q, int lo = 0) {
  int hi = npairs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    lo = (pre[mid * span] <= q) ? mid : lo;
    hi = (pre[mid * span] <= q) ? hi : mid - 1;
  }
  return lo;
}

// One level of pairwise merging over nk variable-length runs whose boundaries
// are pre[0..nk] (pre[nk] = total).  At level `span` (2, 4, 8, ...) the runs
// [pre[p*span], pre[p*span+span/2]) and [pre[p*span+span/2], pre[p*span+span])
// are merged.  Runs may be empty.  A thread whose outputs reach the end of its
// pair continues with the next non-empty pair (rare; a uniform branch).  All
// ITEMS steps run; outputs past the tile end are garbage the caller does not
// write back.
template <int ITEMS, class KeyT, class V, class Cmp>
__device__ __forceinline__ void merge_level_var(const KeyT* sk, const V* sv, const int* pre, int nk, int span,
                                                int s, int e, KeyT (&ok)[ITEMS], V (&ov)[ITEMS], Cmp cmp) {
  (void)e;
  const int npairs = (nk + span - 1) / span;
  int p = find_pair(pre, npairs, span, s);
  int ps = pre[p * span];
  int pm = pre[min(p * span + span / 2, nk)];
  int pe = pre[min(p * span + span, nk)];
  const int diag = s - ps;
  const int ia = merge_path(sk + ps, pm - ps, sk + pm, pe - pm, diag, cmp);
  MergeCursor<KeyT> c;
  c.init(sk, ps + ia, pm, pm + (diag - ia), pe, cmp);
  if (pe - s >= ITEMS) {
    // common case: all ITEMS outputs come from this pair -- no per-step checks
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      int src;
      bool ta;
      ok[i] = c.step(sk, cmp, src, ta);
      if constexpr (HasVal<V>::value) ov[i] = sv[src];
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    if (c.exhausted()) {
      // the pair ends at position s+i == pe: continue in the pair holding it
      const int q = s + i;
      p = find_pair(pre, npairs, span, q, p < npairs - 1 ? p + 1 : p);
      ps = pre[p * span];
      pm = pre[min(p * span + span / 2, nk)];
      pe = pre[min(p * span + span, nk)];
      c.init(sk, ps, pm, pm, pe, cmp);
    }
    int src;
    bool ta;
    ok[i] = c.step(sk, cmp, src, ta);
    if constexpr (HasVal<V>::value) ov[i] = sv[src];
  }
}

// Largest element (under cmp) across the block; every thread gets it.
// `scratch` holds NT keys.  Shared-memory tree, so any copyable key type works
// (no shuffle of user types).
template <int NT, class KeyT, class Cmp>
__device__ __forceinline__ KeyT block_max(KeyT x, KeyT* scratch, Cmp cmp) {
  const int t = threadIdx.x;
  scratch[t] = x;
  __syncthreads();
#pragma unroll
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (t < s) {
      const KeyT a = scratch[t];
      const KeyT b = scratch[t + s];
      scratch[t] = cmp(a, b) ? b : a;
    }
    __syncthreads();
  }
  const KeyT m = scratch[0];
  __syncthreads();
  return m;
}

}  // namespace gms
