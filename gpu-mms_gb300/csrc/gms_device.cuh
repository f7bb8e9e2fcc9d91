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
#include <cstring>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

namespace gms {

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The engine launches its kernels with
// programmatic stream serialization: a kernel's launch is set up while the
// previous kernel of the stream runs, and its CTAs are scheduled as that
// kernel's CTAs exit (no kernel ever triggers its dependents early -- CTAs
// that wait for the rest of a long last wave only take SM slots).  Every such
// kernel calls pdl_wait() before it touches global memory; the wait returns
// once the previous kernel has completed and its writes are visible.  Without
// a programmatic dependency it is a no-op.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

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
// Warp-wide bitonic merging of per-lane sorted runs (keys-only, unstable).
//
// Reference counterpart: merge32..merge512 / merge*dir with __shfl_xor_sync
// (GPU-MMS src/basecase/sortRowMajor.hxx:133-311).  Here each lane holds KPL
// keys sorted ascending in registers, the warp's element e = lane*KPL + r
// (row-major), and five phases merge lane runs into one sorted run of 32*KPL
// keys: phase q merges pairs of runs spread over 2^(q-1) lanes by a mirror
// ("flip") exchange followed by half-cleaners -- across lanes for strides of
// at least KPL elements, inside the lane for smaller ones.  The partner of a
// mirror exchange is register KPL-1-r of lane ^ (2^q - 1); registers r and
// KPL-1-r are exchanged together so only two temporaries are live.
template <class KeyT, class Cmp>
__device__ __forceinline__ KeyT keep_lo_hi(bool lo, const KeyT& a, const KeyT& b, Cmp cmp) {
  // one comparison folded with the lane's side and one select (b is kept by
  // the lower lane when it is smaller, by the upper lane when it is not;
  // equal keys are identical here): uint64 2^27 sort 7.35 -> 6.84 ms on GB300
  // against selecting the minimum or the maximum by side
  const bool take_b = cmp(b, a) ^ !lo;
  return take_b ? b : a;
}

template <int KPL, class KeyT, class Cmp>
__device__ __forceinline__ void warp_merge_runs(KeyT (&x)[KPL], Cmp cmp) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 1; q <= 5; ++q) {
    const int G = 1 << q;
    const bool lower = (lane & (G >> 1)) == 0;
    // mirror exchange with lane ^ (G-1), register KPL-1-r
#pragma unroll
    for (int r = 0; r < KPL / 2; ++r) {
      const KeyT ya = __shfl_xor_sync(0xffffffffu, x[KPL - 1 - r], G - 1);
      const KeyT yb = __shfl_xor_sync(0xffffffffu, x[r], G - 1);
      x[r] = keep_lo_hi(lower, x[r], ya, cmp);
      x[KPL - 1 - r] = keep_lo_hi(lower, x[KPL - 1 - r], yb, cmp);
    }
    // half-cleaners across lanes (element strides 16*G/4 ... KPL)
#pragma unroll
    for (int m = G >> 2; m >= 1; m >>= 1) {
      const bool lo = (lane & m) == 0;
#pragma unroll
      for (int r = 0; r < KPL; ++r) {
        const KeyT z = __shfl_xor_sync(0xffffffffu, x[r], m);
        x[r] = keep_lo_hi(lo, x[r], z, cmp);
      }
    }
    // half-cleaners inside the lane (strides KPL/2 ... 1)
#pragma unroll
    for (int sd = KPL / 2; sd >= 1; sd >>= 1) {
#pragma unroll
      for (int r = 0; r < KPL; ++r) {
        if ((r & sd) == 0) cas(x[r], x[r + sd], cmp);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Shared-memory access through 32-bit shared-window addresses.  For 4- and
// 8-byte keys the loads are explicit ld.shared (no generic 64-bit address
// arithmetic); other types use ordinary accesses.
template <class T>
__device__ __forceinline__ T lds(uint32_t addr) {
  if constexpr (sizeof(T) == 4) {
    uint32_t v;
    asm("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
    T t;
    memcpy(&t, &v, 4);
    return t;
  } else if constexpr (sizeof(T) == 8) {
    unsigned long long v;
    asm("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    T t;
    memcpy(&t, &v, 8);
    return t;
  } else {
    T t;
    // any other size: an ordinary access through a shared pointer
    const unsigned char* p = static_cast<const unsigned char*>(__cvta_shared_to_generic(addr));
    memcpy(&t, p, sizeof(T));
    return t;
  }
}

template <class T>
__device__ __forceinline__ void sts(uint32_t addr, const T& x) {
  if constexpr (sizeof(T) == 4) {
    uint32_t v;
    memcpy(&v, &x, 4);
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
  } else if constexpr (sizeof(T) == 8) {
    unsigned long long v;
    memcpy(&v, &x, 8);
    asm volatile("st.shared.b64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
  } else {
    unsigned char* p = static_cast<unsigned char*>(__cvta_shared_to_generic(addr));
    memcpy(p, &x, sizeof(T));
  }
}

// 16-byte shared store of four 32-bit words (the address 16-byte aligned).
__device__ __forceinline__ void sts_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Loaders.  Keys are addressed by 32-bit shared-window BYTE addresses, so a
// merge step advances a pointer by sizeof(KeyT) and loads at an immediate
// offset, with no index multiply.  PlainLoad reads keys as stored; EncLoad
// applies the codec (a merge reading raw user keys from a staging buffer).
template <class KeyT>
struct PlainLoad {
  uint32_t base;  // shared-window byte address of element 0
  __device__ __forceinline__ explicit PlainLoad(const KeyT* p) : base(static_cast<uint32_t>(__cvta_generic_to_shared(p))) {}
  __device__ __forceinline__ uint32_t addr(int i) const { return base + (uint32_t)i * (uint32_t)sizeof(KeyT); }
  __device__ __forceinline__ KeyT at(uint32_t a) const { return lds<KeyT>(a); }
};
template <class KeyT, class Codec>
struct EncLoad {
  uint32_t base;
  int on;
  __device__ __forceinline__ EncLoad(const KeyT* p, int on_) : base(static_cast<uint32_t>(__cvta_generic_to_shared(p))), on(on_) {}
  __device__ __forceinline__ uint32_t addr(int i) const { return base + (uint32_t)i * (uint32_t)sizeof(KeyT); }
  __device__ __forceinline__ KeyT at(uint32_t a) const {
    const KeyT x = lds<KeyT>(a);
    return on ? Codec::enc(x) : x;
  }
};

// Shared-memory store helper with a fixed base.
template <class T>
struct SmemArray {
  uint32_t base;
  __device__ __forceinline__ explicit SmemArray(const T* p) : base(static_cast<uint32_t>(__cvta_generic_to_shared(p))) {}
  __device__ __forceinline__ void put(int i, const T& x) const { sts<T>(base + (uint32_t)i * (uint32_t)sizeof(T), x); }
  __device__ __forceinline__ T get(int i) const { return lds<T>(base + (uint32_t)i * (uint32_t)sizeof(T)); }
};

// Shared-memory byte address of the payload of the key at byte address `src`,
// keys laid out from `kbase` and payloads from `vbase` at the same element
// indices (src - kbase is a multiple of the key size): one add when key and
// payload have the same size, a shift and an add for 8-byte keys with 4-byte
// payloads.
template <class KeyT, class V>
__device__ __forceinline__ uint32_t payload_addr(uint32_t src, uint32_t kbase, uint32_t vbase) {
  if constexpr (sizeof(KeyT) == sizeof(V)) {
    return src + (vbase - kbase);
  } else if constexpr (sizeof(KeyT) == 2 * sizeof(V)) {
    return vbase + ((src - kbase) >> 1);
  } else {
    return vbase + (src - kbase) / (uint32_t)sizeof(KeyT) * (uint32_t)sizeof(V);
  }
}

// Merge path over [lo, hi]: number of elements of A (byte address a0) among the
// first `diag` outputs of the stable merge of A and B (byte address b0), A
// winning ties, searched only inside [lo, hi].  Branch-free steps.
template <class KeyT, class Ld, class Cmp>
__device__ __forceinline__ int merge_path_in(const Ld& ld, uint32_t a0, uint32_t b0, int diag, int lo, int hi,
                                             Cmp cmp) {
  constexpr uint32_t S = sizeof(KeyT);
  const uint32_t bd = b0 + (uint32_t)(diag - 1) * S;  // B[diag-1-mid] = bd - mid*S
  int len = hi - lo;
  while (len > 0) {
    const int half = len >> 1;
    const int mid = lo + half;
    const bool go = !cmp(ld.at(bd - (uint32_t)mid * S), ld.at(a0 + (uint32_t)mid * S));
    lo = go ? mid + 1 : lo;
    len = go ? len - half - 1 : half;
  }
  return lo;
}

template <class KeyT, class Ld, class Cmp>
__device__ __forceinline__ int merge_path(const Ld& ld, uint32_t a0, int na, uint32_t b0, int nb, int diag, Cmp cmp) {
  const int lo = diag - nb > 0 ? diag - nb : 0;
  const int hi = diag < na ? diag : na;
  return merge_path_in<KeyT>(ld, a0, b0, diag, lo, hi, cmp);
}

// Cursor of a stable two-way merge.  A = [xa, ea), B = [xb, eb) as byte
// addresses; ka/kb are the heads.  step() emits the smaller head (A wins ties)
// and advances that side with one unconditional load right after the consumed
// element (buffers carry slack elements, so it stays in bounds).  No branches.
template <class KeyT>
struct MergeCursor {
  uint32_t xa, ea, xb, eb;
  KeyT ka, kb;

  template <class Ld>
  __device__ __forceinline__ void init(const Ld& ld, uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1) {
    xa = a0;
    ea = a1;
    xb = b0;
    eb = b1;
    ka = ld.at(a0);
    kb = ld.at(b0);
  }

  // Returns the emitted key; `src` receives its byte address, `took_a` its side.
  template <class Ld, class Cmp>
  __device__ __forceinline__ KeyT step(const Ld& ld, Cmp cmp, uint32_t& src, bool& took_a) {
    constexpr uint32_t S = sizeof(KeyT);
    const bool ta = (xb >= eb) || ((xa < ea) && !cmp(kb, ka));
    const KeyT o = ta ? ka : kb;
    const uint32_t cur = ta ? xa : xb;
    const KeyT nv = ld.at(cur + S);
    xa = ta ? cur + S : xa;
    xb = ta ? xb : cur + S;
    ka = ta ? nv : ka;
    kb = ta ? kb : nv;
    src = cur;
    took_a = ta;
    return o;
  }

  // step() for a cursor that cannot run out of either run before it stops:
  // no end checks.
  template <class Ld, class Cmp>
  __device__ __forceinline__ KeyT step_inner(const Ld& ld, Cmp cmp, uint32_t& src, bool& took_a) {
    constexpr uint32_t S = sizeof(KeyT);
    const bool ta = !cmp(kb, ka);
    const KeyT o = ta ? ka : kb;
    const uint32_t cur = ta ? xa : xb;
    const KeyT nv = ld.at(cur + S);
    xa = ta ? cur + S : xa;
    xb = ta ? xb : cur + S;
    ka = ta ? nv : ka;
    kb = ta ? kb : nv;
    src = cur;
    took_a = ta;
    return o;
  }

  __device__ __forceinline__ bool exhausted() const { return xa + xb == ea + eb; }
};

// Cursor of a sentinel-padded two-way merge of keys whose equal keys are
// identical (no end checks, no side bookkeeping).  The two heads are kept
// unordered: a step emits the smaller head, advances the cursor it came from
// and loads that run's next key into slot 1, and moves the other cursor and
// its key (the larger head) into slot 2.  Per step: one comparison, a
// minimum and a maximum of the keys, two address selects, one add and the
// load -- two instructions fewer than tracking which cursor is A and which
// is B.  Ties take slot 1; the emitted values are those of the exact merge
// (equal keys are interchangeable), and a cursor still advances at most once
// per step, so it reads at most one key past the last key it took.
template <class KeyT>
struct MergeCursorSw {
  uint32_t x1, x2;  // byte addresses of the two heads
  KeyT k1, k2;      // the two heads

  template <class Ld>
  __device__ __forceinline__ void init(const Ld& ld, uint32_t a0, uint32_t b0) {
    x1 = a0;
    x2 = b0;
    k1 = ld.at(a0);
    k2 = ld.at(b0);
  }

  template <class Ld, class Cmp>
  __device__ __forceinline__ KeyT step(const Ld& ld, Cmp cmp) {
    constexpr uint32_t S = sizeof(KeyT);
    const bool t = cmp(k2, k1);
    const KeyT o = t ? k2 : k1;
    const KeyT ko = t ? k1 : k2;
    const uint32_t cur = t ? x2 : x1;
    x2 = t ? x1 : x2;
    k2 = ko;
    x1 = cur + S;
    k1 = ld.at(cur + S);
    return o;
  }
};

// One merge pair of a level: its first output position and its two runs
// (element indices into the level's input buffer).
struct PairRange {
  int out0;    // output position of the pair's first element
  int a0, ea;  // run A
  int b0, eb;  // run B
  int id;      // pair index (for payload lookups)
};

// Produces the ITEMS outputs [s, s+ITEMS) of one merge level.
//   pair_of(q)  -> PairRange of the pair holding output position q
//   emit(i, key, src_index, took_a, pair) stores output i
// When all ITEMS outputs lie in one pair (the common case) the thread runs two
// independent merge streams (outputs [s, s+H) and [s+H, s+ITEMS)), so two
// dependency chains are in flight; the second stream's merge-path search only
// scans the H+1 candidates after the first's co-rank.  Otherwise a single
// stream walks across pair ends.  Positions past the valid outputs produce
// garbage that the caller never reads.
template <int ITEMS, class KeyT, class Ld, class Cmp, class PairOf, class Emit>
__device__ __forceinline__ void merge_thread(int s, const Ld& ld, Cmp cmp, const PairOf& pair_of, const Emit& emit) {
  constexpr int H = (ITEMS + 1) / 2;
  constexpr uint32_t S = sizeof(KeyT);
  PairRange P = pair_of(s);
  const int na = P.ea - P.a0, nb = P.eb - P.b0;
  const int diag = s - P.out0;
  uint32_t A0 = ld.addr(P.a0), B0 = ld.addr(P.b0);
  if (na + nb - diag >= ITEMS) {
    const int ia1 = merge_path<KeyT>(ld, A0, na, B0, nb, diag, cmp);
    const int d2 = diag + H;
    int lo2 = d2 - nb > ia1 ? d2 - nb : ia1;
    int hi2 = ia1 + H;
    hi2 = hi2 < na ? hi2 : na;
    hi2 = hi2 < d2 ? hi2 : d2;
    const int ia2 = merge_path_in<KeyT>(ld, A0, B0, d2, lo2, hi2, cmp);
    const uint32_t EA = A0 + (uint32_t)na * S, EB = B0 + (uint32_t)nb * S;
    MergeCursor<KeyT> c1, c2;
    c1.init(ld, A0 + (uint32_t)ia1 * S, EA, B0 + (uint32_t)(diag - ia1) * S, EB);
    c2.init(ld, A0 + (uint32_t)ia2 * S, EA, B0 + (uint32_t)(d2 - ia2) * S, EB);
#pragma unroll
    for (int i = 0; i < H; ++i) {
      uint32_t src1;
      bool ta1;
      const KeyT o1 = c1.step(ld, cmp, src1, ta1);
      emit(i, o1, src1, ta1, P);
      if (H + i < ITEMS) {
        uint32_t src2;
        bool ta2;
        const KeyT o2 = c2.step(ld, cmp, src2, ta2);
        emit(H + i, o2, src2, ta2, P);
      }
    }
    return;
  }
  const int ia = merge_path<KeyT>(ld, A0, na, B0, nb, diag, cmp);
  MergeCursor<KeyT> c;
  c.init(ld, A0 + (uint32_t)ia * S, A0 + (uint32_t)na * S, B0 + (uint32_t)(diag - ia) * S, B0 + (uint32_t)nb * S);
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    if (c.exhausted()) {
      P = pair_of(s + i);
      A0 = ld.addr(P.a0);
      B0 = ld.addr(P.b0);
      c.init(ld, A0, ld.addr(P.ea), B0, ld.addr(P.eb));
    }
    uint32_t src;
    bool ta;
    const KeyT o = c.step(ld, cmp, src, ta);
    emit(i, o, src, ta, P);
  }
}

// Produces outputs [diag, diag + m) of the stable merge of A (byte address a0,
// na keys) and B (b0, nb keys), where 0 < m <= ITEMS and diag + m <= na + nb:
// the window never crosses the end of its pair, so every thread of a warp runs
// the same code.  `lanes` is the mask of the warp's lanes that make this call
// (all of them reach it).  NS independent streams of H = ceil(ITEMS/NS)
// outputs keep NS dependency chains in flight; stream q's merge-path search
// scans only the H+1 candidates after stream q-1's co-rank.
//
// CHECK selects how the steps deal with the ends of the two runs:
//   0  every step checks both run ends; outputs at or past m are computed
//      from in-bounds slack and dropped, never emitted;
//   1  as 0, unless no calling lane can reach a run end within its window
//      and every window is full (a vote over `lanes`, so no divergence):
//      then the steps run without end checks or emit predicates;
//   2  never checked: in shared memory both runs are followed by at least
//      RunPad::read sentinel keys (the largest key under `cmp`), and all ITEMS
//      outputs are emitted, the ITEMS - m past the pair's end into the gap
//      after it.  Merging from an exact co-rank, a window emits the m
//      smallest remaining keys and then, both runs spent, only sentinels, so
//      the emitted values are those of the exact merge and the spill writes
//      sentinels into the gap.  For keys-only merges whose equal keys are
//      identical (the output is fixed by its values); the steps use the
//      unordered cursor MergeCursorSw.
template <int ITEMS, class KeyT, int NS = 2, int CHECK = 1, class Ld, class Cmp, class Emit>
__device__ __forceinline__ void merge_window(const Ld& ld, Cmp cmp, uint32_t A0, int na, uint32_t B0, int nb, int diag,
                                             int m, unsigned lanes, const Emit& emit) {
  constexpr int H = (ITEMS + NS - 1) / NS;
  constexpr uint32_t S = sizeof(KeyT);
  const uint32_t EA = A0 + (uint32_t)na * S, EB = B0 + (uint32_t)nb * S;
  int iq[NS], dq[NS];
  iq[0] = merge_path<KeyT>(ld, A0, na, B0, nb, diag, cmp);
  dq[0] = diag;
#pragma unroll
  for (int q = 1; q < NS; ++q) {
    const int d = diag + q * H < na + nb ? diag + q * H : na + nb;
    const int lo = d - nb > iq[q - 1] ? d - nb : iq[q - 1];
    int hi = iq[q - 1] + H;
    hi = hi < na ? hi : na;
    hi = hi < d ? hi : d;
    iq[q] = merge_path_in<KeyT>(ld, A0, B0, d, lo, hi, cmp);
    dq[q] = d;
  }
  if constexpr (CHECK == 2) {
    MergeCursorSw<KeyT> c[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) c[q].init(ld, A0 + (uint32_t)iq[q] * S, B0 + (uint32_t)(dq[q] - iq[q]) * S);
#pragma unroll
    for (int i = 0; i < H; ++i) {
#pragma unroll
      for (int q = 0; q < NS; ++q) {
        if (q * H + i < ITEMS) {
          const KeyT o = c[q].step(ld, cmp);
          emit(q * H + i, o, 0u, true);
        }
      }
    }
    return;
  }
  MergeCursor<KeyT> c[NS];
#pragma unroll
  for (int q = 0; q < NS; ++q) c[q].init(ld, A0 + (uint32_t)iq[q] * S, EA, B0 + (uint32_t)(dq[q] - iq[q]) * S, EB);
  bool unchecked = false;
  if constexpr (CHECK == 1) {
    bool inner = m == ITEMS;
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      const int hq = ITEMS - q * H < H ? ITEMS - q * H : H;  // outputs of stream q
      inner = inner && na - iq[q] >= hq && nb - (dq[q] - iq[q]) >= hq;
    }
    unchecked = __all_sync(lanes, inner);
  }
  if (unchecked) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
#pragma unroll
      for (int q = 0; q < NS; ++q) {
        if (q * H + i < ITEMS) {
          uint32_t src;
          bool ta;
          const KeyT o = c[q].step_inner(ld, cmp, src, ta);
          emit(q * H + i, o, src, ta);
        }
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < H; ++i) {
#pragma unroll
      for (int q = 0; q < NS; ++q) {
        if (q * H + i < ITEMS) {
          uint32_t src;
          bool ta;
          const KeyT o = c[q].step(ld, cmp, src, ta);
          if (q * H + i < m) emit(q * H + i, o, src, ta);
        }
      }
    }
  }
}

// Keys-only merges under the default order of unsigned stored keys can pad
// every run in shared memory with sentinels (the largest key) and merge
// without end checks (merge_window CHECK 2).
template <class KeyT, class V, class Cmp>
struct SentinelMerge {
  static constexpr bool value =
      !HasVal<V>::value && std::is_same<Cmp, KeyLess>::value && std::is_unsigned<KeyT>::value;
};
// The sentinel of a padded merge: the largest unsigned key (other key types
// are never padded; they get a value-initialised placeholder).
template <class KeyT>
__device__ __forceinline__ constexpr KeyT sentinel_key() {
  if constexpr (std::is_unsigned<KeyT>::value) {
    return (KeyT) ~(KeyT)0;
  } else {
    return KeyT{};
  }
}

// Padding of sentinel-merged runs for windows of ITEMS outputs in NS streams
// (all 0 when the merge checks run ends instead):
//   read  sentinels a window can read past a run's end: a stream of
//         H = ceil(ITEMS/NS) outputs loads the key after each one it takes;
//   gap   keys between consecutive output pairs of a level: room for the
//         ITEMS - 1 outputs a pair's last window spills past the pair's end,
//         and for the next level's `read` sentinels.
template <class KeyT, class V, class Cmp, int ITEMS, int NS>
struct RunPad {
  static constexpr bool on = SentinelMerge<KeyT, V, Cmp>::value;
  static constexpr int read = on ? (ITEMS + NS - 1) / NS + 1 : 0;
  static constexpr int gap = on ? (read > ITEMS - 1 ? read : ITEMS - 1) : 0;
};

// Largest pair index p (< npairs) whose start pre[p*span] is <= q.
__device__ __forceinline__ int find_pair(const int* pre, int npairs, int span, int q) {
  int lo = 0, hi = npairs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const bool le = pre[mid * span] <= q;
    lo = le ? mid : lo;
    hi = le ? hi : mid - 1;
  }
  return lo;
}

// Pair lookup for a level of `span` over compact runs with boundaries pre[].
struct CompactPairs {
  const int* pre;
  int nk, span, npairs;
  __device__ __forceinline__ PairRange operator()(int q) const {
    const int p = find_pair(pre, npairs, span, q);
    const int ps = pre[p * span];
    const int pm = pre[min(p * span + span / 2, nk)];
    const int pe = pre[min(p * span + span, nk)];
    return PairRange{ps, ps, pm, pm, pe, p};
  }
};

// Pair lookup for equal runs of length rl inside a tile of cap keys.
struct RegularPairs {
  int rl, cap;
  __device__ __forceinline__ PairRange operator()(int q) const {
    const int ps = (q / (2 * rl)) * (2 * rl);
    const int pm = min(ps + rl, cap);
    const int pe = min(ps + 2 * rl, cap);
    return PairRange{ps, ps, pm, pm, pe, ps / (2 * rl)};
  }
};

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
