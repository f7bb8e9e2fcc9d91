// Kernels of one multiway-mergesort round on GB300 (sm_103a).
//
// Reference counterparts (GPU-MMS, paths relative to its src/):
//   squareSort            basecase/squareSort.hxx:62-131   -> tile_kernel<MODE_BASE>
//   multimergeLevel       multimergesort.hxx:155-209       -> tile_kernel<MODE_GROUP / MODE_TILE>
//   multimergePipeline    io-merge-gen.hxx:306-355         -> the shared-memory merge levels
//   findPartitions        warp-partition.hxx:488-532       -> splitter_kernel
//   pad                   pad.hxx:1-4                      -> in-kernel tail padding (MODE_BASE)
//
// Layout: one CTA owns one tile of at most CAP = NT*ITEMS keys (+ payload) in
// shared memory.  A tile is loaded with coalesced loads, merged in
// ceil(log2 K) pairwise merge-path levels (results pass through registers and
// back to the same buffer), and stored with coalesced stores.  While storing,
// the CTA also writes every B-th key of its output run (the block sample the
// next round uses to cut its tiles).
#pragma once

#include "gms_device.cuh"
#include "gms_tma.cuh"

namespace gms {

enum TileMode : int { MODE_BASE = 0, MODE_GROUP = 1, MODE_TILE = 2 };

// A group of one round of a segmented (batched) sort.  Groups of such a round
// are listed instead of being K consecutive runs of L keys counted from the
// array start, so that no group crosses a segment: group g covers keys
// [start, start + len) (runs of L keys, the last possibly short), its first
// input run has the global index run0 (block samples of run r sit at
// r * ceil(L / sample_b)), its forecast tiles are [tile0, next tile0), its
// boundary rows [row0, next row0).  flags bit 0: the group reads and writes
// the second buffer pair (in2/out2) of the launch; bit 1: the group's keys are
// decoded as they are stored (its segment's last round).  A list of G groups
// has G + 1 entries; the last one holds the totals (tile0, row0).
// For the base case the groups are the tiles (one run each).
struct GroupDesc {
  int64_t start, len, run0, tile0, row0, flags;
};
enum GroupFlags : int64_t { GRP_ALT = 1, GRP_DEC = 2 };

// Arguments of one launch of tile_kernel.
template <class KeyT, class V>
struct TileArgs {
  const KeyT* in;
  KeyT* out;
  const V* vin;
  V* vout;
  int64_t n;      // elements in the array
  int64_t L;      // input run length (GROUP/TILE); tile length (BASE)
  int k;          // fan-in: runs per group (GROUP/TILE)
  // MODE_TILE: tile boundaries.  Row r of `desc` holds the run-relative start
  // of every run of the group; `doff[r]` is the group-relative output offset.
  const int64_t* desc;
  const int64_t* doff;
  int64_t tiles_full;  // tiles of a full group
  int64_t tiles_last;  // tiles of the last group
  int64_t tile_base;   // merge_tiles_kernel: tile index of block 0 (a launch may cover part of a round)
  int64_t groups;
  // block sample of the output runs (for the next round); null if unused
  KeyT* sample_out;
  int64_t out_run_len;     // length of an output run
  int64_t sample_run_len;  // ceil(out_run_len / sample_b)
  int sample_b;
  int enc_on_load;   // apply Codec::enc to loaded keys
  int dec_on_store;  // apply Codec::dec to stored keys
  int gen_index;     // payload = input position (uint32), ignoring vin
  int* err;          // device status word (bit 0: tile over capacity); may be null
  // segmented rounds: groups listed in grp (null: regular groups), the group
  // of every forecast tile, and the second buffer pair of GRP_ALT groups
  const GroupDesc* grp;
  const int32_t* tile_grp;
  const KeyT* in2;
  KeyT* out2;
  const V* vin2;
  V* vout2;
};

// Bits of the device status word.
enum DeviceStatus : int { DEV_TILE_OVERFLOW = 1, DEV_BAD_SEGMENT = 2, DEV_COPY_TIMEOUT = 4 };

template <class KeyT, class V, int CAP>
struct TileSmemLayout {
  static constexpr bool kHasVal = HasVal<V>::value;
  static constexpr int kMaxK = 32;
  // two ping-pong key buffers (+ payload), each with slack elements
  static constexpr size_t key_bytes = ((sizeof(KeyT) * (CAP + 4) + 15) / 16) * 16;
  static constexpr size_t val_bytes = kHasVal ? ((sizeof(V) * (CAP + 4) + 15) / 16) * 16 : 0;
  static constexpr size_t pre_bytes = 16 * ((sizeof(int) * (kMaxK + 1) + 15) / 16);
  static constexpr size_t gs_bytes = sizeof(int64_t) * kMaxK;
  static constexpr size_t off_k1 = key_bytes;
  static constexpr size_t off_v0 = 2 * key_bytes;
  static constexpr size_t off_v1 = off_v0 + val_bytes;
  static constexpr size_t off_pre = off_v1 + val_bytes;
  static constexpr size_t off_gs = off_pre + pre_bytes;
  static constexpr size_t off_bar = off_gs + gs_bytes;  // mbarrier of the base tile's bulk load
  static constexpr size_t bytes = off_bar + 16;
};

__device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

// Arguments of one group of a segmented round: the buffer pair its flags
// select and, for its segment's last round, decoding on store.
template <class KeyT, class V>
__device__ __forceinline__ void use_group(TileArgs<KeyT, V>& a, int64_t flags) {
  if (flags & GRP_ALT) {
    a.in = a.in2;
    a.out = a.out2;
    a.vin = a.vin2;
    a.vout = a.vout2;
  }
  if (flags & GRP_DEC) a.dec_on_store = 1;
}

template <class Codec, class KeyT>
__device__ __forceinline__ KeyT maybe_enc(KeyT x, int on) {
  return on ? Codec::enc(x) : x;
}
template <class Codec, class KeyT>
__device__ __forceinline__ KeyT maybe_dec(KeyT x, int on) {
  return on ? Codec::dec(x) : x;
}

// Keys per 16-byte vector, and the position of a global key pointer within
// its 16-byte line (in keys).  A tile whose last merge level writes its output
// `vec_shift(g)` keys into a 16-byte-aligned shared buffer has its shared and
// global keys 16-byte aligned at the same indices, so it can be stored with
// 16-byte loads and stores (store_tile).
template <class KeyT>
struct VecKeys {
  static constexpr int E = 16 / (int)sizeof(KeyT);
  static constexpr bool on = sizeof(KeyT) == 4 || sizeof(KeyT) == 8;
};
template <class KeyT>
__device__ __forceinline__ int vec_shift(const KeyT* g) {
  return (int)((reinterpret_cast<uintptr_t>(g) / sizeof(KeyT)) % VecKeys<KeyT>::E);
}

// Stores the keys f[0, cnt) of shared memory to g[0, cnt) of global memory,
// decoded when `dec`, by threads t0, t0 + nthr, ... of the CTA: 16-byte loads
// and stores between the first and the last 16-byte boundary of g, single
// keys at the two ends.  f must sit vec_shift(g) keys past a 16-byte boundary
// (and g be aligned to its key size).
template <class Codec, class KeyT>
__device__ __forceinline__ void store_tile(const KeyT* f, KeyT* g, int cnt, int dec, int t0, int nthr) {
  constexpr int E = VecKeys<KeyT>::E;
  const int mis = vec_shift(g);
  const int h = min(cnt, (E - mis) % E);  // keys before g's first 16-byte boundary
  const int nvec = (cnt - h) / E;
  const int tail0 = h + nvec * E;
  const int nscal = h + (cnt - tail0);
  for (int j = t0; j < nscal; j += nthr) {
    const int q = j < h ? j : tail0 + (j - h);
    g[q] = maybe_dec<Codec>(f[q], dec);
  }
  const uint4* fv = reinterpret_cast<const uint4*>(f + h);
  uint4* gv = reinterpret_cast<uint4*>(g + h);
  if (dec) {
    for (int v = t0; v < nvec; v += nthr) {
      uint4 w = fv[v];
      if constexpr (sizeof(KeyT) == 4) {
        w.x = Codec::dec(w.x);
        w.y = Codec::dec(w.y);
        w.z = Codec::dec(w.z);
        w.w = Codec::dec(w.w);
      } else {
        const uint64_t lo = Codec::dec((uint64_t)w.x | ((uint64_t)w.y << 32));
        const uint64_t hi = Codec::dec((uint64_t)w.z | ((uint64_t)w.w << 32));
        w = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
      }
      gv[v] = w;
    }
  } else {
    for (int v = t0; v < nvec; v += nthr) gv[v] = fv[v];
  }
}

// Comparator on raw user bits that encodes both sides first (when `on`).
template <class Cmp, class Codec>
struct EncCmp {
  int on;
  template <class KeyT>
  __device__ __forceinline__ bool operator()(const KeyT& x, const KeyT& y) const {
    return Cmp()(maybe_enc<Codec>(x, on), maybe_enc<Codec>(y, on));
  }
};

// ---------------------------------------------------------------------------
// The tile kernel.
//   MODE_BASE : tile t covers [t*L, t*L+L) with L <= CAP.  Keys are sorted in
//               registers (ITEMS per thread), then merged in shared memory up
//               to the whole tile.  A short last tile is padded with copies of
//               its own largest key, which sort after every real key, so no
//               sentinel value is reserved.
//   MODE_GROUP: CTA g merges the K runs of group g (K*L <= CAP).
//   MODE_TILE : CTA merges one tile of a group whose runs are cut by `desc`.
// STABLE: equivalent keys keep their input order (used for key/value sorts and
// for user comparators whose equivalent keys may differ in their bits).
// With a.grp (segmented rounds) CTA g takes group g: MODE_BASE sorts the tile
// [start, start + len), MODE_GROUP merges the group's runs; MODE_TILE is not
// used with listed groups.
template <class KeyT, class V, class Cmp, class Codec, int MODE, bool STABLE, int NT, int ITEMS>
__global__ void __launch_bounds__(NT, (MODE == MODE_BASE && sizeof(KeyT) == 4 && !HasVal<V>::value) ? 3 : 1)
    tile_kernel(TileArgs<KeyT, V> a0) {
  pdl_wait();
  TileArgs<KeyT, V> a = a0;
  const GroupDesc* gd = a.grp ? a.grp + blockIdx.x : nullptr;
  if (gd) use_group(a, gd->flags);
  constexpr int CAP = NT * ITEMS;
  constexpr bool kHasVal = HasVal<V>::value;
  using Lay = TileSmemLayout<KeyT, V, CAP>;
  extern __shared__ __align__(16) unsigned char smem[];
  KeyT* const k0 = reinterpret_cast<KeyT*>(smem);
  KeyT* const k1 = reinterpret_cast<KeyT*>(smem + Lay::off_k1);
  V* const v0 = reinterpret_cast<V*>(smem + Lay::off_v0);
  V* const v1 = reinterpret_cast<V*>(smem + Lay::off_v1);
  int* pre = reinterpret_cast<int*>(smem + Lay::off_pre);
  int64_t* gs = reinterpret_cast<int64_t*>(smem + Lay::off_gs);
  const Cmp cmp;
  const int tid = threadIdx.x;
  KeyT* sk = k0;
  V* sv = v0;

  int64_t out_base;   // global index of this tile's first output
  int64_t run_base;   // global index of the output run this tile belongs to
  int64_t run_index;  // index of that output run
  int cnt;            // keys in this tile
  int nk = 1;         // runs in the tile (GROUP/TILE)
  int cur = 0;        // buffer holding the current level's input
  const int s = tid * ITEMS;

  if constexpr (MODE == MODE_BASE) {
    const int64_t base = gd ? gd->start : (int64_t)blockIdx.x * a.L;
    if (base >= a.n) return;
    cnt = gd ? (int)gd->len : (int)min64(a.L, a.n - base);
    out_base = base;
    run_base = base;
    run_index = blockIdx.x;
    KeyT r[ITEMS];
    V rv[ITEMS];
    if constexpr (STABLE) {
      // Stable: each thread must own a contiguous chunk of the input, so the
      // input is staged through shared memory -- by bulk copies (TMA) for a
      // full tile at 16-byte-aligned addresses, else by striped loads.
      bool bulk = cnt == CAP && (reinterpret_cast<uint64_t>(a.in + base) & 15) == 0;
      const bool copy_v = kHasVal && !a.gen_index;
      if constexpr (kHasVal) bulk = bulk && (!copy_v || (reinterpret_cast<uint64_t>(a.vin + base) & 15) == 0);
      if (bulk) {
        uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Lay::off_bar);
        int* timed_out = pre;
        if (tid == 0) {
          const uint32_t kb = (uint32_t)(CAP * sizeof(KeyT));
          const uint32_t vb = copy_v ? (uint32_t)(CAP * sizeof(V)) : 0u;
          mbar_init(bar, 1);
          fence_mbar_init();
          mbar_arrive_expect_tx(bar, kb + vb);
          bulk_g2s(sk, a.in + base, kb, bar);
          if constexpr (kHasVal) {
            if (copy_v) bulk_g2s(sv, a.vin + base, vb, bar);
          }
        }
        if (tid < 32) {
          constexpr uint32_t kSpinLimit = 1u << 26;
          __syncwarp();
          const bool ok = mbar_wait_bounded(bar, 0, kSpinLimit);
          if ((tid & 31) == 0) *timed_out = ok ? 0 : 1;
          if (!ok) {
            if ((tid & 31) == 0 && a.err) atomicOr(a.err, DEV_COPY_TIMEOUT);
            // let the copies in flight land (a second timeout returns anyway: the
            // status bit already marks the result invalid)
            mbar_wait_bounded(bar, 0, kSpinLimit);
          }
        }
        __syncthreads();
        if (*timed_out) return;
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
          const int p = tid * ITEMS + i;
          r[i] = maybe_enc<Codec>(sk[p], a.enc_on_load);
          if constexpr (kHasVal) rv[i] = copy_v ? sv[p] : (V)(base + p);
        }
      } else {
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
          const int p = tid + i * NT;
          if (p < cnt) {
            sk[p] = maybe_enc<Codec>(a.in[base + p], a.enc_on_load);
            if constexpr (kHasVal) sv[p] = a.gen_index ? (V)(base + p) : a.vin[base + p];
          }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
          const int p = tid * ITEMS + i;
          r[i] = sk[p < cnt ? p : 0];
          if constexpr (kHasVal) rv[i] = sv[p < cnt ? p : 0];
        }
      }
      if (cnt < CAP) {
        KeyT m = r[0];
#pragma unroll
        for (int i = 1; i < ITEMS; ++i) {
          if (tid * ITEMS + i < cnt) m = cmp(m, r[i]) ? r[i] : m;
        }
        __syncthreads();  // every chunk is in registers; the buffer is free as scratch
        m = block_max<NT>(m, sk, cmp);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
          if (tid * ITEMS + i >= cnt) r[i] = m;
        }
      }
      transposition_sort<ITEMS>(r, rv, cmp);
      __syncthreads();
    } else {
      // Coalesced striped load: register i of thread t holds element t + i*NT.
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const int p = tid + i * NT;
        if (p < cnt) r[i] = maybe_enc<Codec>(a.in[base + p], a.enc_on_load);
      }
      if (cnt < CAP) {
        // a short last tile is padded with copies of its largest key
        KeyT m = r[0];
        if (tid >= cnt) m = maybe_enc<Codec>(a.in[base], a.enc_on_load);
#pragma unroll
        for (int i = 1; i < ITEMS; ++i) {
          if (tid + i * NT < cnt) m = cmp(m, r[i]) ? r[i] : m;
        }
        m = block_max<NT>(m, sk, cmp);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
          if (tid + i * NT >= cnt) r[i] = m;
        }
      }
      network_sort<ITEMS>(r, cmp);
    }
    // Blocked write: thread t's sorted run at [t*ITEMS, t*ITEMS+ITEMS).
    // ITEMS is odd, so the ITEMS-strided stores hit distinct banks.
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      sk[s + i] = r[i];
      if constexpr (kHasVal) sv[s + i] = rv[i];
    }
    __syncthreads();
    // Merge levels up to the whole (padded) tile, ping-ponging the buffers.
    // Runs of rl = ITEMS * 2^lv keys: pair p (2 * rl keys) gets exactly
    // 2 * rl / ITEMS threads, so every window is full and none crosses a
    // pair's end (window-aligned merges, no pair lookup per output).
    static_assert((NT & (NT - 1)) == 0, "the base tile's merge levels need a power-of-two thread count");
    for (int rl = ITEMS; rl < CAP; rl *= 2) {
      const KeyT* xk = (cur ? k1 : k0);
      KeyT* yk = (cur ? k0 : k1);
      const V* xv = (cur ? v1 : v0);
      V* yv = (cur ? v0 : v1);
      const PlainLoad<KeyT> ld(xk);
      const SmemArray<KeyT> yka(yk + s);
      const SmemArray<V> yva(yv + s);
      const uint32_t xvb = static_cast<uint32_t>(__cvta_generic_to_shared(xv));
      const int tpp = 2 * rl / ITEMS;
      const int p = tid / tpp;
      const int diag = (tid - p * tpp) * ITEMS;
      const int ps = p * 2 * rl;
      merge_window<ITEMS, KeyT, 2, 1>(ld, cmp, ld.addr(ps), rl, ld.addr(ps + rl), rl, diag, ITEMS, 0xffffffffu,
                                      [&](int i, KeyT k, uint32_t src, bool) {
                                        yka.put(i, k);
                                        if constexpr (kHasVal) yva.put(i, lds<V>(payload_addr<KeyT, V>(src, ld.base, xvb)));
                                      });
      __syncthreads();
      cur ^= 1;
    }
  } else {
    // ---- GROUP / TILE: gather the K input segments into shared memory ----
    int64_t gbase;
    int64_t tile_off = 0;  // group-relative output offset
    int64_t g;
    if constexpr (MODE == MODE_GROUP) {
      g = blockIdx.x;
      gbase = gd ? gd->start : g * a.L * a.k;
      if (gbase >= a.n) return;
      const int64_t ng = gd ? gd->len : min64(a.L * a.k, a.n - gbase);
      cnt = (int)ng;
      nk = a.k;
      if (tid <= nk) pre[tid] = (int)min64((int64_t)tid * a.L, ng);
      const KeyT* src = a.in + gbase;
      for (int p = tid; p < cnt; p += NT) {
        sk[p] = maybe_enc<Codec>(src[p], a.enc_on_load);
        if constexpr (kHasVal) sv[p] = a.gen_index ? (V)(gbase + p) : a.vin[gbase + p];
      }
    } else {
      const int64_t tau = blockIdx.x;
      g = tau / a.tiles_full;
      const int64_t j = tau - g * a.tiles_full;
      const int64_t jg = (g == a.groups - 1) ? a.tiles_last : a.tiles_full;
      if (j >= jg) return;
      gbase = g * a.L * a.k;
      const int64_t row = g * (a.tiles_full + 1) + j;
      nk = a.k;
      const int64_t ng = min64(a.L * a.k, a.n - gbase);
      if (tid < 32) {
        int len = 0;
        if (tid < nk) {
          const int64_t lo = a.desc[row * nk + tid];
          const int64_t hi = a.desc[(row + 1) * nk + tid];
          // a segment must lie inside its run and hold at most CAP keys
          const int64_t rl = min64(a.L, ng - min64((int64_t)tid * a.L, ng));
          const bool ok_seg = (lo >= 0) && (hi >= lo) && (hi <= rl) && (hi - lo <= CAP);
          len = ok_seg ? (int)(hi - lo) : 0;
          if (!ok_seg) {
            len = CAP + 1;  // forces the capacity check below to reject the tile
            if (a.err) atomicOr(a.err, DEV_BAD_SEGMENT);
          }
          gs[tid] = gbase + (int64_t)tid * a.L + lo;
        }
        // inclusive scan of segment lengths across the warp
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (tid >= o) incl += y;
        }
        if (tid < nk) pre[tid + 1] = incl;
        if (tid == 0) pre[0] = 0;
      }
      tile_off = a.doff[row];
      __syncthreads();
      cnt = pre[nk];
      if (cnt > CAP || cnt < 0) {
        // never overrun the shared-memory tile: report and skip
        if (tid == 0 && a.err) atomicOr(a.err, DEV_TILE_OVERFLOW);
        return;
      }
      for (int kk = 0; kk < nk; ++kk) {
        const int b = pre[kk];
        const int len = pre[kk + 1] - b;
        const int64_t src = gs[kk];
        for (int i = tid; i < len; i += NT) {
          sk[b + i] = maybe_enc<Codec>(a.in[src + i], a.enc_on_load);
          if constexpr (kHasVal) sv[b + i] = a.gen_index ? (V)(src + i) : a.vin[src + i];
        }
      }
    }
    out_base = gbase + tile_off;
    run_base = gbase;
    run_index = g;
    __syncthreads();
    // ---- ceil(log2 nk) levels of pairwise merging, ping-ponging ----
    for (int span = 2; span < 2 * nk; span *= 2) {
      const KeyT* xk = (cur ? k1 : k0);
      KeyT* yk = (cur ? k0 : k1);
      const V* xv = (cur ? v1 : v0);
      V* yv = (cur ? v0 : v1);
      if (s < cnt) {
        const PlainLoad<KeyT> ld(xk);
        const SmemArray<KeyT> yka(yk + s);
        const SmemArray<V> yva(yv + s);
        const uint32_t xvb = static_cast<uint32_t>(__cvta_generic_to_shared(xv));
        const CompactPairs pairs{pre, nk, span, (nk + span - 1) >> (31 - __clz(span))};
        merge_thread<ITEMS, KeyT>(s, ld, cmp, pairs, [&](int i, KeyT k, uint32_t src, bool, const PairRange&) {
          yka.put(i, k);
          if constexpr (kHasVal) yva.put(i, lds<V>(payload_addr<KeyT, V>(src, ld.base, xvb)));
        });
      }
      __syncthreads();
      cur ^= 1;
    }
  }

  // ---- coalesced store of the merged tile (+ block sample) ----
  const KeyT* fk = (cur ? k1 : k0);
  const V* fv = (cur ? v1 : v0);
  for (int p = tid; p < cnt; p += NT) {
    a.out[out_base + p] = maybe_dec<Codec>(fk[p], a.dec_on_store);
    if constexpr (kHasVal) a.vout[out_base + p] = fv[p];
  }
  if (a.sample_out) {
    // output positions whose offset in the output run is a multiple of B
    const int64_t rel0 = out_base - run_base;
    const int64_t first = (a.sample_b - rel0 % a.sample_b) % a.sample_b;
    for (int64_t p = first + (int64_t)tid * a.sample_b; p < cnt; p += (int64_t)NT * a.sample_b) {
      a.sample_out[run_index * a.sample_run_len + (rel0 + p) / a.sample_b] = fk[p];
    }
  }
}

// ---------------------------------------------------------------------------
// Base case for keys-only sorts of 4- and 8-byte keys: register network per
// lane, warp-shuffle bitonic merges up to one 32*KPL-key run per warp, then
// shared-memory merge-path levels up to the TILE = NT*KPL-key tile.
//
// Reference counterpart: squareSort (GPU-MMS src/basecase/squareSort.hxx:62-131)
// with its register sort (bitonicSort32) and shuffle merges (merge32..512).
template <int NT, int KPL, int ITEMS_M, int PAD_ = 0>
struct BaseWarpGeom {
  static constexpr int PAD = PAD_;  // sentinel slots after every run in shared memory (0: none)
  static constexpr int TILE = NT * KPL;
  static constexpr int WARP_RUN = 32 * KPL;
  static constexpr int log2i(int x) { return x <= 1 ? 0 : 1 + log2i(x / 2); }
  static constexpr int LEVELS = log2i(TILE / WARP_RUN);  // shared-memory merge levels
  static_assert((WARP_RUN << LEVELS) == TILE, "TILE must be WARP_RUN times a power of two");
  // the windows of the first level (pairs of WARP_RUN keys) must fit the block
  static constexpr int WINDOWS = (TILE / (2 * WARP_RUN)) * ((2 * WARP_RUN + ITEMS_M - 1) / ITEMS_M);
  static_assert(LEVELS == 0 || WINDOWS <= NT, "merge windows exceed the block");
  static_assert((KPL & (KPL - 1)) == 0 && KPL % 4 == 0, "KPL must be a power of two, multiple of 4");
};

// Each ping-pong buffer holds the tile plus slack for the reads past a pair's
// end of the last window of a pair (at most ITEMS_M/2 + 2 keys), and with
// sentinel padding a gap of PAD keys after every run.
template <class KeyT, int NT, int KPL, int ITEMS_M, int PAD = 0>
struct BaseWarpSmem {
  using Geo = BaseWarpGeom<NT, KPL, ITEMS_M, PAD>;
  static constexpr int SPAN = Geo::TILE + (Geo::TILE / Geo::WARP_RUN) * PAD + ITEMS_M;
  static constexpr size_t buf = ((sizeof(KeyT) * (SPAN + 4) + 15) / 16) * 16;
  static constexpr size_t off_bar = 2 * buf;  // mbarrier of the tile's bulk load
  static constexpr size_t bytes = off_bar + 16;
};

// Runs in shared memory are padded with PAD sentinel keys (the largest key)
// when the order allows it (RunPad), so the merge levels step without run-end
// checks; the pad after each run is refilled at every level.
// With a.grp (segmented sorts) CTA t sorts the tile [start, start + len) of
// group (tile) t.
template <class KeyT, class Cmp, class Codec, int NT, int KPL, int ITEMS_M, int NSB = 2>
__global__ void __launch_bounds__(NT) base_warp_kernel(TileArgs<KeyT, NoVal> a0) {
  pdl_wait();
  TileArgs<KeyT, NoVal> a = a0;
  const GroupDesc* gd = a.grp ? a.grp + blockIdx.x : nullptr;
  if (gd) use_group(a, gd->flags);
  constexpr int PAD = RunPad<KeyT, NoVal, Cmp, ITEMS_M, NSB>::gap;
  using Geo = BaseWarpGeom<NT, KPL, ITEMS_M, PAD>;
  constexpr int TILE = Geo::TILE;
  constexpr size_t BUF = BaseWarpSmem<KeyT, NT, KPL, ITEMS_M, PAD>::buf;
  extern __shared__ __align__(16) unsigned char smem[];
  KeyT* const k0 = reinterpret_cast<KeyT*>(smem);
  KeyT* const k1 = reinterpret_cast<KeyT*>(smem + BUF);
  const Cmp cmp;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int64_t base = gd ? gd->start : (int64_t)blockIdx.x * TILE;
  if (base >= a.n) return;
  const int cnt = gd ? (int)gd->len : (int)min64(TILE, a.n - base);

  // Load: register i of thread t holds element t + i*NT.  A full tile at a
  // 16-byte-aligned address arrives by one bulk copy (TMA) into the second
  // buffer and is read from there (one copy engine request instead of KPL
  // loads per thread); otherwise coalesced loads straight from global memory.
  KeyT x[KPL];
  const bool bulk = cnt == TILE && (reinterpret_cast<uint64_t>(a.in + base) & 15) == 0;
  if (bulk) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + BaseWarpSmem<KeyT, NT, KPL, ITEMS_M, PAD>::off_bar);
    int* timed_out = reinterpret_cast<int*>(smem) + 0;  // k0[0], free until the warp runs are stored
    if (tid == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
      mbar_arrive_expect_tx(bar, (uint32_t)(TILE * sizeof(KeyT)));
      bulk_g2s(k1, a.in + base, (uint32_t)(TILE * sizeof(KeyT)), bar);
    }
    if (tid < 32) {
      constexpr uint32_t kSpinLimit = 1u << 26;
      __syncwarp();
      const bool ok = mbar_wait_bounded(bar, 0, kSpinLimit);
      if (lane == 0) *timed_out = ok ? 0 : 1;
      if (!ok) {
        if (lane == 0 && a.err) atomicOr(a.err, DEV_COPY_TIMEOUT);
        // let the copies in flight land (a second timeout returns anyway: the
        // status bit already marks the result invalid)
        mbar_wait_bounded(bar, 0, kSpinLimit);
      }
    }
    __syncthreads();
    if (*timed_out) return;
#pragma unroll
    for (int i = 0; i < KPL; ++i) x[i] = maybe_enc<Codec>(k1[tid + i * NT], a.enc_on_load);
    __syncthreads();  // k0[0] and k1 are reused below
  } else {
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
      const int p = tid + i * NT;
      if (p < cnt) x[i] = maybe_enc<Codec>(a.in[base + p], a.enc_on_load);
    }
  }
  if (cnt < TILE) {
    // a short last tile is padded with copies of its largest key
    KeyT m = x[0];
    if (tid >= cnt) m = maybe_enc<Codec>(a.in[base], a.enc_on_load);
#pragma unroll
    for (int i = 1; i < KPL; ++i) {
      if (tid + i * NT < cnt) m = cmp(m, x[i]) ? x[i] : m;
    }
    m = block_max<NT>(m, k0, cmp);
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
      if (tid + i * NT >= cnt) x[i] = m;
    }
  }
  network_sort<KPL>(x, cmp);
  warp_merge_runs<KPL>(x, cmp);
  // The warp's sorted run: lane l holds elements l*KPL .. l*KPL+KPL-1.  With
  // padding, run w starts at w*(WARP_RUN + PAD) and is followed by PAD
  // sentinels.
  {
    KeyT* run = k0 + warp * (Geo::WARP_RUN + PAD);
    constexpr int KPC = 16 / (int)sizeof(KeyT);  // keys per 16-byte chunk
    constexpr int NC = KPL / KPC;                // chunks per lane
    if constexpr (NC >= 8 && NC % 8 == 0 && ((Geo::WARP_RUN + PAD) * sizeof(KeyT)) % 16 == 0) {
      // A lane's run is a multiple of 128 bytes, so the same store of every
      // lane would hit the same banks.  Lane l writes its chunk c ^ (l & 7)
      // at step c instead: the eight lanes of a quarter-warp then write eight
      // different bank groups (conflict-free 16-byte stores).  The chunks
      // are XOR-permuted in registers first (three conditional swaps).
      const int t = lane & 7;
#pragma unroll
      for (int b = 1; b < 8; b <<= 1) {
        const bool sw = (t & b) != 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if ((c & b) == 0) {
#pragma unroll
            for (int e = 0; e < KPC; ++e) {
              const KeyT u = x[c * KPC + e], v = x[(c ^ b) * KPC + e];
              x[c * KPC + e] = sw ? v : u;
              x[(c ^ b) * KPC + e] = sw ? u : v;
            }
          }
        }
      }
      const uint32_t base =
          static_cast<uint32_t>(__cvta_generic_to_shared(run)) + (uint32_t)(KPL * sizeof(KeyT)) * (uint32_t)lane;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        uint32_t w[4];
        memcpy(w, &x[c * KPC], 16);
        sts_v4(base + 16u * (uint32_t)(c ^ t), w[0], w[1], w[2], w[3]);
      }
    } else {
      const SmemArray<KeyT> dst(run + lane * KPL);
#pragma unroll
      for (int r = 0; r < KPL; ++r) dst.put(r, x[r]);
    }
    if constexpr (PAD > 0) {
      for (int j = lane; j < PAD; j += 32) run[Geo::WARP_RUN + j] = sentinel_key<KeyT>();
    }
  }
  __syncthreads();
  // shared-memory merge levels: runs of WARP_RUN ... TILE/2.  Each pair of a
  // level gets ceil(2*rl/ITEMS_M) threads whose windows never cross its end.
  int cur = 0;
#pragma unroll
  for (int lv = 0; lv < Geo::LEVELS; ++lv) {
    const int rl = Geo::WARP_RUN << lv;
    const int tpp = (2 * rl + ITEMS_M - 1) / ITEMS_M;
    const int np = TILE / (2 * rl);
    const KeyT* xk = cur ? k1 : k0;
    KeyT* yk = cur ? k0 : k1;
    const unsigned lanes = __ballot_sync(0xffffffffu, tid < tpp * np);
    if (tid < tpp * np) {
      const int p = tid / tpp;
      const int diag = (tid - p * tpp) * ITEMS_M;
      const int m = min(ITEMS_M, 2 * rl - diag);
      const PlainLoad<KeyT> ld(xk);
      // input runs 2p and 2p+1 (length rl, PAD apart); output pair p
      const SmemArray<KeyT> yka(yk + p * (2 * rl + PAD) + diag);
      merge_window<ITEMS_M, KeyT, NSB, (PAD > 0 ? 2 : 0)>(
          ld, cmp, ld.addr(2 * p * (rl + PAD)), rl, ld.addr((2 * p + 1) * (rl + PAD)), rl, diag, m, lanes,
          [&](int i, KeyT k, uint32_t, bool) { yka.put(i, k); });
    }
    if constexpr (PAD > 0) {
      // sentinels after every output pair, read by the next level (the
      // windows that end a pair spill the same value into the gap)
      if (lv + 1 < Geo::LEVELS) {
        for (int x2 = tid; x2 < np * PAD; x2 += NT) {
          const int p = x2 / PAD;
          yk[p * (2 * rl + PAD) + 2 * rl + (x2 - p * PAD)] = sentinel_key<KeyT>();
        }
      }
    }
    __syncthreads();
    cur ^= 1;
  }
  // coalesced store (+ block sample of the output run = this tile)
  const KeyT* fk = cur ? k1 : k0;
  for (int p = tid; p < cnt; p += NT) a.out[base + p] = maybe_dec<Codec>(fk[p], a.dec_on_store);
  if (a.sample_out) {
    for (int p = tid * a.sample_b; p < cnt; p += NT * a.sample_b) {
      a.sample_out[(int64_t)blockIdx.x * a.sample_run_len + p / a.sample_b] = fk[p];
    }
  }
}

// ---------------------------------------------------------------------------
// K-way merge of one forecast tile per CTA, staged with bulk copies.
//
// Warp 0 places the K run segments of the tile in the staging buffer
// (16-byte-aligned regions) and issues one cp.async.bulk per segment,
// completing on an mbarrier transaction count.  The first merge level reads
// the staged segment pairs directly; the remaining ceil(log2 K)-1 levels
// ping-pong between the merge buffer and the (now free) staging buffer.  Three
// CTAs of 512 threads fit an SM for 4-byte keys, so one CTA's copy latency is
// covered by the others' merging.
// With sentinel padding (RunPad: READ sentinels after each staged segment,
// GAP keys after each output pair of a level) the buffers are sized by the
// tile limit TMAX plus the padding instead of by CAP.
template <class KeyT, class V, int CAP, int SETS = 1, int READ = 0, int GAP = 0, int TMAX = CAP, int ITEMS = 0>
struct MergeSmemLayout {
  static constexpr bool kHasVal = HasVal<V>::value;
  static constexpr int kMaxK = 32;
  static constexpr size_t round16(size_t x) { return (x + 15) / 16 * 16; }
  // every segment region may add up to 30 bytes of alignment slack; a padded
  // segment's region holds its keys and READ sentinels from a start at most 12
  // bytes into its first 16, rounded up to 16
  static constexpr size_t stage_k_bytes =
      READ ? round16(sizeof(KeyT) * TMAX + kMaxK * (sizeof(KeyT) * READ + 27) + 16)
           : round16(sizeof(KeyT) * (CAP + 4) + 32 * kMaxK + 16);
  static constexpr size_t stage_v_bytes = kHasVal ? round16(sizeof(V) * (CAP + 4) + 32 * kMaxK + 16) : 0;
  // the merge buffer takes the even levels' outputs: up to kMaxK/2 pairs, GAP
  // apart, and the last window's spill of up to ITEMS - 1 keys
  static constexpr size_t mk_bytes =
      READ ? round16(sizeof(KeyT) * (TMAX + (kMaxK / 2) * GAP + ITEMS + 4)) : round16(sizeof(KeyT) * (CAP + 4));
  static constexpr size_t mv_bytes = kHasVal ? round16(sizeof(V) * (CAP + 4)) : 0;
  static constexpr size_t off_stage_v = stage_k_bytes;
  static constexpr size_t off_mk = off_stage_v + stage_v_bytes;
  static constexpr size_t off_mv = off_mk + mk_bytes;
  // SETS descriptor sets, one per tile in flight: cpre[33] int, sbk[32] int,
  // sbv[32] int, a status word, gsrc[32] int64, meta[6] int64, wst[kLevels][17]
  // int (first thread of each pair's windows, per level); then the mbarrier.
  static constexpr int kLevels = 5;  // log2(kMaxK)
  static constexpr size_t set_gsrc = 400;
  static constexpr size_t set_meta = set_gsrc + 8 * 32;
  static constexpr size_t set_wst = set_meta + 8 * 6;
  static constexpr size_t set_bytes = round16(set_wst + 4 * kLevels * 17);
  static constexpr size_t off_desc = off_mv + mv_bytes;
  static constexpr size_t off_bar = off_desc + SETS * set_bytes;
  static constexpr size_t bytes = off_bar + 16;
};

// Merge-tile capacity with window-aligned levels: at a level with np pairs
// the windows of ITEMS outputs that never cross a pair end number at most
// cnt/ITEMS + np, which fits NT threads when cnt <= (NT - kMaxK/2) * ITEMS.
template <int NT, int ITEMS>
struct WindowCap {
  static constexpr int value = (NT - 16) * ITEMS;
};

// One descriptor set in shared memory (see MergeSmemLayout).
struct TileDesc {
  int* cpre;      // segment prefix: segment s is keys [cpre[s], cpre[s+1]) of the tile
  int* sbk;       // element index of segment s in the staged keys
  int* sbv;       // ... in the staged payload
  int* status;    // 1: the copy wait timed out
  int64_t* gsrc;  // global index of segment s's first key
  int64_t* meta;  // output offset, run base, run index, key count (-1: rejected), group flags
  int* wst;       // window tables
  __device__ __forceinline__ TileDesc(unsigned char* base, size_t set_gsrc, size_t set_meta, size_t set_wst)
      : cpre(reinterpret_cast<int*>(base)),
        sbk(cpre + 33),
        sbv(sbk + 32),
        status(cpre + 97),
        gsrc(reinterpret_cast<int64_t*>(base + set_gsrc)),
        meta(reinterpret_cast<int64_t*>(base + set_meta)),
        wst(reinterpret_cast<int*>(base + set_wst)) {}
};

// COPY selects how a tile's segments reach shared memory: 1 = warp 0 issues
// one cp.async.bulk per segment (mbarrier completion); 2 = every warp
// computes the placement and copies a share of the segments with 16-byte
// cp.async (group completion), which spreads the issue over all warps.
// PERSIST (with COPY 1): each CTA loops over tiles blockIdx.x + i*gridDim.x;
// when the merged tile ends in the merge buffer, warp 0 stages the next tile
// into the free staging buffer while the other warps store the current one.
template <class KeyT, class V, class Cmp, int NT, int ITEMS, int NS, bool PERSIST>
using MergeLayoutOf =
    MergeSmemLayout<KeyT, V, NT * ITEMS, PERSIST ? 2 : 1, RunPad<KeyT, V, Cmp, ITEMS, NS>::read,
                    RunPad<KeyT, V, Cmp, ITEMS, NS>::gap, WindowCap<NT, ITEMS>::value, ITEMS>;

// Keys-only merges under the default order pad every run with sentinels
// (RunPad): staged segment s is followed by READ sentinels in its region, and
// level outputs are laid out with a gap of PAD keys after every pair (pair p
// of a level starts at cpre[first segment] + p*PAD), refilled with sentinels
// at every level, so the merge steps never check run ends (merge_window CHECK
// 2).  Without padding (payload merges, user comparators) the steps check.
// Each instantiation is compiled for the CTAs per SM that its shared memory
// allows (228 KB per SM, 1 KB reserved per CTA; at most 3), so its register
// budget never lowers that residency.  Left to itself the compiler chose, for
// the same source, 40 registers and spills for the 288 x 31 keys-only merge,
// and 92 registers -- two CTAs per SM instead of three -- for the persistent
// 288 x 15 float32 + int32 merge.
template <class Lay>
struct MergeMinBlocks {
  static constexpr int by_smem = (int)((228u * 1024u) / (Lay::bytes + 1024u));
  static constexpr int value = by_smem < 1 ? 1 : (by_smem > 3 ? 3 : by_smem);
};
template <class KeyT, class V, class Cmp, class Codec, int NT, int ITEMS, int NS, int COPY = 1, bool PERSIST = false>
__global__ void __launch_bounds__(NT, (MergeMinBlocks<MergeLayoutOf<KeyT, V, Cmp, NT, ITEMS, NS, PERSIST>>::value))
    merge_tiles_kernel(TileArgs<KeyT, V> a, int64_t total_tiles) {
  static_assert(!PERSIST || COPY == 1, "persistent tiles stage with bulk copies");
  pdl_wait();
  constexpr int CAP = NT * ITEMS;                        // shared-memory buffers
  constexpr int TILE_MAX = WindowCap<NT, ITEMS>::value;  // keys a tile may hold
  constexpr bool kHasVal = HasVal<V>::value;
  constexpr int READ = RunPad<KeyT, V, Cmp, ITEMS, NS>::read;
  constexpr int PAD = RunPad<KeyT, V, Cmp, ITEMS, NS>::gap;
  using Lay = MergeLayoutOf<KeyT, V, Cmp, NT, ITEMS, NS, PERSIST>;
  static_assert(Lay::off_desc % 16 == 0 && Lay::set_gsrc % 8 == 0, "descriptor alignment");
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* stage_k = smem;
  unsigned char* stage_v = smem + Lay::off_stage_v;
  KeyT* const k0 = reinterpret_cast<KeyT*>(stage_k);
  KeyT* const k1 = reinterpret_cast<KeyT*>(smem + Lay::off_mk);
  V* const v0 = reinterpret_cast<V*>(stage_v);
  V* const v1 = reinterpret_cast<V*>(smem + Lay::off_mv);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Lay::off_bar);
  const Cmp cmp;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int nk = a.k;
  auto desc_set = [&](int s) {
    return TileDesc(smem + Lay::off_desc + (size_t)s * Lay::set_bytes, Lay::set_gsrc, Lay::set_meta, Lay::set_wst);
  };
  // tiles of this launch: [a.tile_base, total_tiles); indices past a group's
  // last tile are empty
  auto real_tile = [&](int64_t t) {
    if (a.grp) return true;  // listed groups: tiles are numbered without gaps
    const int64_t g = t / a.tiles_full;
    const int64_t j = t - g * a.tiles_full;
    return j < ((g == a.groups - 1) ? a.tiles_last : a.tiles_full);
  };
  // tile t's group, boundary row, keys and group flags
  struct TileLoc {
    int64_t g, row, gbase, ng, flags;
  };
  auto locate = [&](int64_t t) {
    TileLoc l;
    if (a.grp) {
      l.g = a.tile_grp[t];
      const GroupDesc& gd = a.grp[l.g];
      l.row = gd.row0 + (t - gd.tile0);
      l.gbase = gd.start;
      l.ng = gd.len;
      l.flags = gd.flags;
    } else {
      l.g = t / a.tiles_full;
      l.row = l.g * (a.tiles_full + 1) + (t - l.g * a.tiles_full);
      l.gbase = l.g * a.L * a.k;
      l.ng = min64(a.L * a.k, a.n - l.gbase);
      l.flags = 0;
    }
    return l;
  };
  auto next_tile = [&](int64_t t) {
    if (!PERSIST) return total_tiles;
    for (t += gridDim.x; t < total_tiles && !real_tile(t); t += gridDim.x) {
    }
    return t < total_tiles ? t : total_tiles;
  };
  int64_t tau = a.tile_base + blockIdx.x;
  if (tau >= total_tiles) return;
  if (!real_tile(tau)) {
    tau = next_tile(tau);
    if (tau >= total_tiles) return;
  }

  if constexpr (COPY == 1) {
    if (tid == 0) mbar_init(bar, 1);
    fence_mbar_init();
    __syncthreads();
  }

  // ---- place tile t's segments in the staging buffer and issue their copies
  // (warp 0; every warp with COPY 2), filling descriptor set d.  Ordered to
  // start the copies early: the descriptor and output-offset loads go out
  // together, the two prefix sums that place the segments run side by side,
  // and the bookkeeping the merge levels need (segment starts, window tables)
  // is written while the copies are in flight.
  // A tile's boundary row (lane s: run s's first and end offsets; lane 0 also
  // the tile's output offset), loaded ahead of its use.
  struct Bounds {
    int64_t lo = 0, hi = 0, out_off = 0;
  };
  auto load_bounds = [&](int64_t t) {
    Bounds b;
    const int64_t row = locate(t).row;
    if (lane < nk) {
      b.lo = a.desc[row * nk + lane];
      b.hi = a.desc[(row + 1) * nk + lane];
    }
    if (lane == 0) b.out_off = a.doff[row];
    return b;
  };
  auto stage = [&](int64_t t, const TileDesc& d, const Bounds& bd) {
    const TileLoc loc = locate(t);
    const int64_t g = loc.g;
    const int64_t gbase = loc.gbase;
    const int64_t ng = loc.ng;
    const bool alt = (loc.flags & GRP_ALT) != 0;
    const KeyT* kin = alt ? a.in2 : a.in;
    const V* vin = alt ? a.vin2 : a.vin;
    const uint64_t arr_k_lo = reinterpret_cast<uint64_t>(kin);
    const uint64_t arr_k_hi = arr_k_lo + (uint64_t)a.n * sizeof(KeyT);
    const int64_t lo = bd.lo, hi = bd.hi, out_off = bd.out_off;
    int len = 0;
    int64_t gs = 0;
    bool bad = false;
    if (lane < nk) {
      const int64_t rl = min64(a.L, ng - min64((int64_t)lane * a.L, ng));
      bad = !((lo >= 0) && (hi >= lo) && (hi <= rl) && (hi - lo <= TILE_MAX));
      len = bad ? 0 : (int)(hi - lo);
      gs = gbase + (int64_t)lane * a.L + (bad ? 0 : lo);
    }
    // key regions
    const uint64_t A = arr_k_lo + (uint64_t)gs * sizeof(KeyT);
    const uint64_t E = A + (uint64_t)len * sizeof(KeyT);
    const SegCopy ck = seg_copy(A, E, arr_k_lo, arr_k_hi);
    uint32_t reg_k = (uint32_t)(ck.e16 - ck.a16);
    if constexpr (READ > 0) {
      // room for the segment's sentinels after its last key
      const uint32_t need = ((uint32_t)(A - ck.a16) + (uint32_t)(len + READ) * (uint32_t)sizeof(KeyT) + 15u) & ~15u;
      if (lane < nk && need > reg_k) reg_k = need;
    }
    int incl = len;
    uint32_t off_k = reg_k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      const uint32_t z = __shfl_up_sync(0xffffffffu, off_k, o);
      if (lane >= o) {
        incl += y;
        off_k += z;
      }
    }
    off_k -= reg_k;  // exclusive
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const bool any_bad = __any_sync(0xffffffffu, bad) || total > TILE_MAX;
    uint32_t bulk = (!any_bad && ck.be > ck.bs) ? (uint32_t)(ck.be - ck.bs) : 0u;
    SegCopy cv{};
    uint32_t off_v = 0;
    uint64_t Av = 0;
    const bool carry = kHasVal && !a.gen_index;
    if constexpr (kHasVal) {
      if (carry) {
        const uint64_t arr_v_lo = reinterpret_cast<uint64_t>(vin);
        const uint64_t arr_v_hi = arr_v_lo + (uint64_t)a.n * sizeof(V);
        Av = arr_v_lo + (uint64_t)gs * sizeof(V);
        const uint64_t Ev = Av + (uint64_t)len * sizeof(V);
        cv = seg_copy(Av, Ev, arr_v_lo, arr_v_hi);
        const uint32_t reg_v = (uint32_t)(cv.e16 - cv.a16);
        off_v = reg_v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, off_v, o);
          if (lane >= o) off_v += y;
        }
        off_v -= reg_v;
        if (!any_bad && cv.be > cv.bs) bulk += (uint32_t)(cv.be - cv.bs);
      }
    }
    if constexpr (COPY == 1) {
      uint32_t tx = bulk;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tx += __shfl_xor_sync(0xffffffffu, tx, o);
      fence_proxy_async_smem();
      if (lane == 0) mbar_arrive_expect_tx(bar, tx);
      __syncwarp();
      if (!any_bad && lane < nk && len > 0) {
        if (ck.be > ck.bs) {
          bulk_g2s(stage_k + off_k + (ck.bs - ck.a16), reinterpret_cast<const void*>(ck.bs), (uint32_t)(ck.be - ck.bs),
                   bar);
        }
        if constexpr (kHasVal) {
          if (carry && cv.be > cv.bs) {
            bulk_g2s(stage_v + off_v + (cv.bs - cv.a16), reinterpret_cast<const void*>(cv.bs),
                     (uint32_t)(cv.be - cv.bs), bar);
          }
        }
      }
    } else {
      // segment s goes to warp s % (NT/32); its lanes copy 16-byte chunks
      (void)bulk;
      if (!any_bad) {
        for (int sg = warp; sg < nk; sg += NT / 32) {
          const uint64_t bs = __shfl_sync(0xffffffffu, ck.bs, sg);
          const uint64_t be = __shfl_sync(0xffffffffu, ck.be, sg);
          const uint64_t a16 = __shfl_sync(0xffffffffu, ck.a16, sg);
          const uint32_t ok = __shfl_sync(0xffffffffu, off_k, sg);
          const int nch = be > bs ? (int)((be - bs) >> 4) : 0;
          unsigned char* dst = stage_k + ok + (uint32_t)(bs - a16);
          for (int c = lane; c < nch; c += 32) cp_async16(dst + 16 * c, reinterpret_cast<const void*>(bs + 16ull * c));
          if constexpr (kHasVal) {
            if (carry) {
              const uint64_t vbs = __shfl_sync(0xffffffffu, cv.bs, sg);
              const uint64_t vbe = __shfl_sync(0xffffffffu, cv.be, sg);
              const uint64_t va16 = __shfl_sync(0xffffffffu, cv.a16, sg);
              const uint32_t ov = __shfl_sync(0xffffffffu, off_v, sg);
              const int nvc = vbe > vbs ? (int)((vbe - vbs) >> 4) : 0;
              unsigned char* vdst = stage_v + ov + (uint32_t)(vbs - va16);
              for (int c = lane; c < nvc; c += 32)
                cp_async16(vdst + 16 * c, reinterpret_cast<const void*>(vbs + 16ull * c));
            }
          }
        }
      }
    }
    if (warp == 0 && !any_bad && lane < nk && len > 0) {
      unsigned char* dstk = stage_k + off_k;
      // plain loads for bytes outside the array's 16-byte-aligned interior
      // (never more than 15 bytes at each end of the array)
      const KeyT* src = kin + gs;
      KeyT* dst = reinterpret_cast<KeyT*>(dstk + (A - ck.a16));
      for (int i = 0; i < len; ++i) {
        const uint64_t addr = A + (uint64_t)i * sizeof(KeyT);
        if (ck.be > ck.bs && addr >= ck.bs && addr < ck.be) {
          i += (int)((ck.be - addr) / sizeof(KeyT)) - 1;  // skip the bulk interior
        } else {
          dst[i] = src[i];
        }
      }
      if constexpr (kHasVal) {
        if (carry) {
          unsigned char* dstv = stage_v + off_v;
          const V* vsrc = vin + gs;
          V* vdst = reinterpret_cast<V*>(dstv + (Av - cv.a16));
          for (int i = 0; i < len; ++i) {
            const uint64_t addr = Av + (uint64_t)i * sizeof(V);
            if (cv.be > cv.bs && addr >= cv.bs && addr < cv.be) {
              i += (int)((cv.be - addr) / sizeof(V)) - 1;
            } else {
              vdst[i] = vsrc[i];
            }
          }
        }
      }
    }
    // bookkeeping for the merge levels, written while the copies fly
    if (warp == 0 && lane < nk) {
      d.cpre[lane + 1] = incl;
      d.sbk[lane] = (int)((off_k + (uint32_t)(A - ck.a16)) / sizeof(KeyT));
      d.gsrc[lane] = gs;
      if (carry) d.sbv[lane] = (int)((off_v + (uint32_t)(Av - cv.a16)) / sizeof(V));
    }
    if (warp == 0 && lane == 0) {
      d.cpre[0] = 0;
      d.meta[0] = gbase + out_off;
      d.meta[1] = gbase;
      d.meta[2] = g;
      d.meta[3] = any_bad ? -1 : total;
      d.meta[4] = loc.flags;
      if (any_bad && a.err) atomicOr(a.err, DEV_BAD_SEGMENT);
    }
    // window table of every level: pair p of a level with `span` segments
    // holds keys [cpre[p*span], cpre[min(p*span+span, nk)]) and gets
    // ceil(len/ITEMS) threads starting at wst[lev*17 + p]
    for (int lev = 0, span = 2; lev < Lay::kLevels && (lev == 0 || (span >> 1) < nk); ++lev, span <<= 1) {
      const int np = (nk + span - 1) / span;
      const int si = lane * span;
      const int ei = min(si + span, nk);
      const int ps = __shfl_sync(0xffffffffu, incl, max(min(si, nk) - 1, 0));
      const int pe = __shfl_sync(0xffffffffu, incl, max(ei - 1, 0));
      const int plen = (lane < np) ? (si == 0 ? pe : pe - ps) : 0;
      const int tcount = (plen + ITEMS - 1) / ITEMS;
      int tincl = tcount;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, tincl, o);
        if (lane >= o) tincl += y;
      }
      if (warp == 0 && lane < np) d.wst[lev * 17 + lane + 1] = tincl;
      if (warp == 0 && lane == 0) d.wst[lev * 17] = 0;
    }
  };

  if (COPY == 2 || warp == 0) stage(tau, desc_set(0), load_bounds(tau));
  int set = 0;
  uint32_t parity = 0;
  while (true) {
    const TileDesc d = desc_set(set);
    // ---- wait for the staged segments (bounded) ----
    // Only warp 0 polls the mbarrier; the other warps wait in the block
    // barrier, which issues nothing.  The barrier orders warp 0's acquire of
    // the copied bytes (and its own plain stores) before every other thread's
    // reads.
    constexpr uint32_t kSpinLimit = 1u << 26;
    // sentinels after every staged segment (the raw-key image of the largest
    // key when the staged keys are encoded as they are read); written after
    // the copies land, since a segment's copy may cover its first pad slots
    // (a rejected tile -- meta[3] < 0 -- has no placement to pad: skipped)
    auto pad_segments = [&](int l0, int lstep) {
      if constexpr (READ > 0) {
        if (d.meta[3] < 0) return;
        const KeyT sv = a.enc_on_load ? Codec::dec(sentinel_key<KeyT>()) : sentinel_key<KeyT>();
        KeyT* sk = reinterpret_cast<KeyT*>(stage_k);
        for (int s = 0; s < nk; ++s) {
          const int e = d.sbk[s] + (d.cpre[s + 1] - d.cpre[s]);
          for (int j = l0; j < READ; j += lstep) sk[e + j] = sv;
        }
      }
    };
    if constexpr (COPY == 1) {
      if (warp == 0) {
        const bool ok = mbar_wait_bounded(bar, parity, kSpinLimit);
        if (lane == 0) *d.status = ok ? 0 : 1;
        if (!ok) {
          if (lane == 0 && a.err) atomicOr(a.err, DEV_COPY_TIMEOUT);
          // let copies in flight land; should this wait run out as well, the CTA
          // still returns -- accepted only because the status bit already marks
          // the sort's result as invalid
          mbar_wait_bounded(bar, parity, kSpinLimit);
        } else {
          __syncwarp();  // lane 0's descriptor writes are visible to the warp
          pad_segments(lane, 32);
        }
      }
    } else {
      cp_async_wait_all();
      if (tid == 0) *d.status = 0;
      if constexpr (READ > 0) {
        __syncthreads();  // every warp's copies have landed
        pad_segments(tid, NT);
      }
    }
    __syncthreads();
    if (*d.status) return;
    const int cnt = (int)d.meta[3];
    if (cnt < 0) return;  // rejected tile (never expected): nothing was copied
    const int64_t out_base = d.meta[0];
    const int64_t run_base = d.meta[1];
    const int64_t run_index = d.meta[2];
    const int* cpre = d.cpre;
    const int* sbk = d.sbk;
    const int* sbv = d.sbv;
    const int64_t* gsrc = d.gsrc;
    // a persistent CTA loads the next tile's boundary row now, so the loads
    // complete during this tile's merge levels
    const int64_t nxt = next_tile(tau);
    Bounds nb_next;
    if (PERSIST && warp == 0 && nxt < total_tiles) nb_next = load_bounds(nxt);
    // Keys-only sentinel-padded merges store the merged tile with 16-byte
    // accesses: the last level writes its output vs keys into the buffer, vs
    // being the output's position within its 16-byte line in global memory.
    constexpr bool kVecStore = !kHasVal && PAD > 0 && VecKeys<KeyT>::on;
    const int vs = kVecStore ? vec_shift(((d.meta[4] & GRP_ALT) ? a.out2 : a.out) + out_base) : 0;

    // ---- levels: window-aligned merges, pair by pair ----
    // Level 0 merges staged segment pairs (2p, 2p+1) into the merge buffer;
    // the later levels ping-pong between the merge buffer and the staging
    // buffer, pair p of level `lev` merging the outputs of pairs 2p and 2p+1
    // below.
    int cur = 0;  // 0: the staging buffer holds the current input
    for (int lev = 0, span = 2; lev == 0 || (span >> 1) < nk; ++lev, span <<= 1) {
      const int np = (nk + span - 1) / span;
      const int* wt = d.wst + lev * 17;
      const unsigned lanes = __ballot_sync(0xffffffffu, tid < wt[np]);
      if (tid < wt[np]) {
        int p = 0;  // the last pair whose first window thread is <= tid
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          if (p + step < np && wt[p + step] <= tid) p += step;
        }
        const int si = p * span;
        const int mi = min(si + (span >> 1), nk);
        const int ei = min(si + span, nk);
        const int ps = cpre[si], pm = cpre[mi], pe = cpre[ei];
        const int diag = (tid - wt[p]) * ITEMS;
        const int m = min(ITEMS, pe - ps - diag);
        const int na = pm - ps, nb = pe - pm;
        // this pair's output (PAD apart from the previous pair; the last
        // level's single pair starts vs keys in)
        const int yo = ps + p * PAD + (span >= nk ? vs : 0);
        constexpr int kCheck = PAD > 0 ? 2 : 1;
        if (lev == 0) {
          // the staged keys are encoded while read only when the round's input
          // is raw caller data (a uniform branch: two specialised loops)
          auto level0 = [&](const auto& ld) {
            const uint32_t A0 = ld.addr(sbk[si]);
            const bool has_b = si + 1 < nk;
            const uint32_t B0 = has_b ? ld.addr(sbk[si + 1]) : A0 + (uint32_t)na * sizeof(KeyT);
            const SmemArray<KeyT> yka(k1 + yo + diag);
            const SmemArray<V> yva(v1 + yo + diag);
            const int gen = a.gen_index;
            // per run of the pair: where its staged payloads start (vA, vB:
            // in the order of its staged keys from A0, B0) and the global
            // index of its first key (gA, gB: generated payloads)
            uint32_t vA = 0, vB = 0, gA = 0, gB = 0;
            if constexpr (kHasVal) {
              const uint32_t vbase = static_cast<uint32_t>(__cvta_generic_to_shared(stage_v));
              vA = vbase + (uint32_t)sbv[si] * (uint32_t)sizeof(V);
              vB = has_b ? vbase + (uint32_t)sbv[si + 1] * (uint32_t)sizeof(V) : vA;
              gA = (uint32_t)gsrc[si];
              gB = has_b ? (uint32_t)gsrc[si + 1] : gA;
            }
            merge_window<ITEMS, KeyT, NS, kCheck>(ld, cmp, A0, na, B0, nb, diag, m, lanes,
                                                  [&](int i, KeyT k, uint32_t src, bool ta) {
                                            yka.put(i, k);
                                            if constexpr (kHasVal) {
                                              const uint32_t s0 = ta ? A0 : B0;
                                              if (gen) {
                                                const uint32_t idx = (src - s0) / (uint32_t)sizeof(KeyT);
                                                yva.put(i, (V)((ta ? gA : gB) + idx));
                                              } else {
                                                yva.put(i, lds<V>(payload_addr<KeyT, V>(src, s0, ta ? vA : vB)));
                                              }
                                            }
                                          });
          };
          if (a.enc_on_load) {
            level0(EncLoad<KeyT, Codec>(reinterpret_cast<const KeyT*>(stage_k), 1));
          } else {
            level0(PlainLoad<KeyT>(reinterpret_cast<const KeyT*>(stage_k)));
          }
        } else {
          const KeyT* xk = (cur ? k1 : k0);
          KeyT* yk = (cur ? k0 : k1);
          const V* xv = (cur ? v1 : v0);
          V* yv = (cur ? v0 : v1);
          const PlainLoad<KeyT> ld(xk);
          const SmemArray<KeyT> yka(yk + yo + diag);
          const SmemArray<V> yva(yv + yo + diag);
          const uint32_t xvb = static_cast<uint32_t>(__cvta_generic_to_shared(xv));
          // input runs: the outputs of pairs 2p and 2p+1 of the level below
          const uint32_t A0 = ld.addr(ps + 2 * p * PAD);
          const uint32_t B0 = mi < nk ? ld.addr(pm + (2 * p + 1) * PAD) : A0 + (uint32_t)na * sizeof(KeyT);
          merge_window<ITEMS, KeyT, NS, kCheck>(ld, cmp, A0, na, B0, nb, diag, m, lanes,
                                                [&](int i, KeyT k, uint32_t src, bool) {
                                                  yka.put(i, k);
                                                  if constexpr (kHasVal)
                                                    yva.put(i, lds<V>(payload_addr<KeyT, V>(src, ld.base, xvb)));
                                                });
        }
      }
      if constexpr (PAD > 0) {
        // sentinels after every output pair, read by the next level (the
        // windows that end a pair spill the same value into the gap)
        if (span < nk) {
          KeyT* yk = (cur ? k0 : k1);
          for (int x = tid; x < np * PAD; x += NT) {
            const int q = x / PAD;
            yk[cpre[min(q * span + span, nk)] + q * PAD + (x - q * PAD)] = sentinel_key<KeyT>();
          }
        }
      }
      __syncthreads();
      cur ^= 1;
    }
    // ---- coalesced store (+ block sample for the next round); in a
    // persistent CTA whose merged tile is in the merge buffer, warp 0 stages
    // the next tile meanwhile ----
    const bool overlap = PERSIST && nxt < total_tiles && cur == 1;
    if (overlap && warp == 0) stage(nxt, desc_set(set ^ 1), nb_next);
    const int t0 = overlap ? tid - 32 : tid;
    const int nthr = overlap ? NT - 32 : NT;
    if (t0 >= 0) {
      const KeyT* fk = (cur ? k1 : k0) + vs;
      const V* fv = (cur ? v1 : v0);
      const int64_t tflags = d.meta[4];
      KeyT* kout = (tflags & GRP_ALT) ? a.out2 : a.out;
      V* vout = (tflags & GRP_ALT) ? a.vout2 : a.vout;
      const int dec = a.dec_on_store | ((tflags & GRP_DEC) ? 1 : 0);
      if constexpr (kVecStore) {
        store_tile<Codec>(fk, kout + out_base, cnt, dec, t0, nthr);
      } else {
        for (int q = t0; q < cnt; q += nthr) {
          kout[out_base + q] = maybe_dec<Codec>(fk[q], dec);
          if constexpr (kHasVal) vout[out_base + q] = fv[q];
        }
      }
      if (a.sample_out) {
        const int64_t rel0 = out_base - run_base;
        const int64_t first = (a.sample_b - rel0 % a.sample_b) % a.sample_b;
        for (int64_t q = first + (int64_t)t0 * a.sample_b; q < cnt; q += (int64_t)nthr * a.sample_b) {
          a.sample_out[run_index * a.sample_run_len + (rel0 + q) / a.sample_b] = fk[q];
        }
      }
    }
    if (nxt >= total_tiles) return;
    __syncthreads();  // the store has read the merged tile before it is overwritten
    if (!overlap && warp == 0) stage(nxt, desc_set(set ^ 1), nb_next);
    tau = nxt;
    set ^= 1;
    parity ^= 1;
  }
}

// ---------------------------------------------------------------------------
// Splitter: exact tile boundaries of one merge round.
//
// For group g the merged block sample F (the first key of every B-key block of
// every run, merged in (key, run, block) order) is cut every G entries.  The
// first key of block F[j*G] is boundary j.  One warp per boundary; lane k finds
// how many keys of run k precede the boundary in the stable (key, run, index)
// order: first the number of run k's blocks whose first key precedes the
// boundary -- which brackets the answer to one block -- then inside that block
// of the run.  The block count is one more than the block index of run k's
// last entry in F before position j*G: the warp scans F's index stream
// backwards from there, 32 entries per coalesced load, until every run has
// shown up (uniform keys: a few loads), the group's sample starts, or
// kScanChunks loads are spent (or two loads show no other run, as in sorted
// stretches); a run not seen by then binary-searches its block sample `samp`
// instead.  Between two boundaries every run contributes
// at most (its blocks in that stretch of F + 1) blocks, so a tile holds at
// most (G + K) * B keys.
// Segmented rounds (grp set): row r belongs to group row_grp[r]; the group's
// runs, block samples and merged sample follow its GroupDesc, and GRP_ALT
// groups read `data2`.
// direct = 1 (a tuning alternative): each lane binary-searches its whole run
// for the boundary key, as the reference's findPartitions does
// (warp-partition.hxx:488-532), instead of first bracketing the answer to one
// block with the run's block sample.
template <class KeyT, class Cmp, class Codec>
__global__ void __launch_bounds__(256) splitter_kernel(const KeyT* __restrict__ data, const KeyT* __restrict__ samp,
                                                        const KeyT* __restrict__ fkeys,
                                                        const uint32_t* __restrict__ fidx, int64_t n, int64_t L,
                                                        int k, int64_t sample_run_len, int sample_b, int64_t G,
                                                        int64_t tiles_full, int64_t tiles_last, int64_t groups,
                                                        int64_t* __restrict__ desc, int64_t* __restrict__ doff,
                                                        int enc, const GroupDesc* __restrict__ grp,
                                                        const int32_t* __restrict__ row_grp,
                                                        const KeyT* __restrict__ data2, int direct) {
  pdl_wait();
  const Cmp cmp;
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t g, j, jg, gbase, ng, run0;
  if (grp) {
    if (row >= grp[groups].row0) return;
    g = row_grp[row];
    const GroupDesc& gd = grp[g];
    j = row - gd.row0;
    jg = grp[g + 1].tile0 - gd.tile0;
    gbase = gd.start;
    ng = gd.len;
    run0 = gd.run0;
    if (gd.flags & GRP_ALT) data = data2;
  } else {
    const int64_t rows_per_group = tiles_full + 1;
    g = row / rows_per_group;
    if (g >= groups) return;
    j = row - g * rows_per_group;
    jg = (g == groups - 1) ? tiles_last : tiles_full;
    if (j > jg) return;
    gbase = g * L * k;
    ng = min64(L * k, n - gbase);
    run0 = g * (int64_t)k;
  }
  // block counts from F's index stream (all lanes of the warp take part)
  constexpr int kScanChunks = 8;  // 32-entry chunks of F a boundary scans at most
  __shared__ int32_t scan_slot[8][32];
  int32_t* slot = scan_slot[(threadIdx.x >> 5) & 7];
  const bool inner = j > 0 && j < jg;
  const int64_t fbase = run0 * sample_run_len;
  const int64_t fpos = fbase + j * G;
  int64_t kb = -1;
  int64_t scan_lo = -1;  // this lane's run: block count found by the scan
  if (inner) {
    kb = (int64_t)fidx[fpos] / sample_run_len - run0;
    if (!direct) {
      // runs with keys (an empty run has no entry to find: its count is 0)
      const bool has_keys = lane < k && min64((int64_t)lane * L, ng) < min64((int64_t)(lane + 1) * L, ng);
      unsigned pending = __ballot_sync(0xffffffffu, has_keys) & ~(1u << (unsigned)kb);
      const unsigned pending0 = pending;
      int64_t q0 = fpos;
      for (int step = 0; step < kScanChunks && pending && q0 > fbase; ++step) {
        // skewed stretches of F (sorted runs, long ties): when the first two
        // chunks show no other run, leave the rest to the block-sample search
        if (step == 2 && pending == pending0) break;
        q0 -= 32;
        const int64_t q = q0 + lane;
        int r = -1, bi = 0;
        if (q >= fbase) {
          const uint32_t si = fidx[q];
          const uint32_t rr = si / (uint32_t)sample_run_len;
          r = (int)((int64_t)rr - run0);
          bi = (int)(si - rr * (uint32_t)sample_run_len);
        }
        // the highest lane of each run's group holds that run's latest entry
        const unsigned same = __match_any_sync(0xffffffffu, r);
        const bool latest = r >= 0 && r < 32 && (same >> lane) == 1u;
        if (latest) slot[r] = bi + 1;
        const unsigned seen = __reduce_or_sync(0xffffffffu, latest ? (1u << r) : 0u);
        __syncwarp();
        if (lane < k && ((seen & pending) >> lane) & 1u) scan_lo = slot[lane];
        pending &= ~seen;
        __syncwarp();
      }
      // reached the group's first sample entry: runs not seen have no block before the boundary
      if (q0 <= fbase && lane < k && ((pending >> lane) & 1u)) scan_lo = 0;
    }
  }
  int64_t c = 0;
  if (lane < k) {
    const int64_t rs = min64((int64_t)lane * L, ng);
    const int64_t re = min64((int64_t)(lane + 1) * L, ng);
    const int64_t len = re - rs;
    if (j == 0) {
      c = 0;
    } else if (j == jg) {
      c = len;
    } else {
      const KeyT v = fkeys[fpos];
      const int64_t sidx = (int64_t)fidx[fpos];
      const int64_t ib = (sidx - (run0 + kb) * sample_run_len) * sample_b;
      if (lane == kb) {
        c = ib;
      } else {
        // earlier runs win ties: a key precedes the boundary if key <= v
        // (lane < kb) or key < v (lane > kb)
        const bool le = lane < kb;
        auto precedes = [=](const KeyT& x) -> bool { return le ? !cmp(v, x) : cmp(x, v); };
        if (direct) {
          const KeyT* r = data + gbase + rs;
          int64_t a0 = 0, a1 = len;
          while (a0 < a1) {
            const int64_t mid = (a0 + a1) >> 1;
            if (precedes(maybe_enc<Codec>(r[mid], enc))) a0 = mid + 1; else a1 = mid;
          }
          c = a0;
        } else {
          // 1. blocks whose first key precedes the boundary (from the scan,
          // else by binary search over the run's block sample)
          int64_t lo = scan_lo;
          if (lo < 0) {
            const KeyT* sr = samp + (run0 + lane) * sample_run_len;
            const int64_t nb = (len + sample_b - 1) / sample_b;
            int64_t hi = nb;
            lo = 0;
            while (lo < hi) {
              const int64_t mid = (lo + hi) >> 1;
              if (precedes(sr[mid])) lo = mid + 1; else hi = mid;
            }
          }
          // 2. inside the last such block
          if (lo == 0) {
            c = 0;
          } else {
            const KeyT* r = data + gbase + rs;
            int64_t a0 = (lo - 1) * sample_b + 1;
            int64_t a1 = min64(lo * (int64_t)sample_b, len);
            while (a0 < a1) {
              const int64_t mid = (a0 + a1) >> 1;
              if (precedes(maybe_enc<Codec>(r[mid], enc))) a0 = mid + 1; else a1 = mid;
            }
            c = a0;
          }
        }
      }
    }
    desc[row * k + lane] = c;
  }
  // group-relative output offset of the tile that starts at this boundary
  int64_t sum = c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) doff[row] = sum;
}

// ---------------------------------------------------------------------------
// Block sample of a sample: out[r*out_run + b] = in[r*in_run + b*B] for every
// run r and every b < ceil(len_r / B).  Run lengths: in_run each, the last
// one up to n_in; or, for segmented rounds, run_len[r].
template <class KeyT, class Codec>
__global__ void gather_sample_kernel(const KeyT* __restrict__ in, KeyT* __restrict__ out, int64_t n_in, int64_t in_run,
                                     int64_t out_run, int b_step, int64_t n_out_slots, int enc,
                                     const int32_t* __restrict__ run_len) {
  pdl_wait();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_out_slots) return;
  const int64_t r = t / out_run;
  const int64_t b = t - r * out_run;
  const int64_t src = r * in_run + b * b_step;
  const int64_t rend = run_len ? r * in_run + run_len[r] : min64((r + 1) * in_run, n_in);
  if (src < rend) out[t] = maybe_enc<Codec>(in[src], enc);
}

// Exact co-ranks at arbitrary output ranks of one K-way task, given the task
// merged with its origin index.  Lane k counts the keys of run k that precede
// or equal the rank-th smallest element (stable order).  Mirrors the contract
// of findPartitions (warp-partition.hxx:488-532) for caller-chosen ranks.
template <class KeyT, class Cmp, class Codec>
__global__ void corank_kernel(const KeyT* __restrict__ task, const KeyT* __restrict__ merged,
                              const uint32_t* __restrict__ origin, int64_t size, int k, int64_t task_size,
                              const int64_t* __restrict__ ranks, int64_t nranks, int64_t* __restrict__ out) {
  const Cmp cmp;
  const int lane = threadIdx.x & 31;
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nranks) return;
  int64_t r = ranks[q];
  r = r < 0 ? 0 : (r > task_size ? task_size : r);
  for (int kk = lane; kk < k; kk += 32) {
    const int64_t rs = min64((int64_t)kk * size, task_size);
    const int64_t re = min64((int64_t)(kk + 1) * size, task_size);
    int64_t c = 0;
    if (r > 0) {
      const KeyT v = merged[r - 1];
      const int64_t o = (int64_t)origin[r - 1];
      const int64_t kb = o / size;
      if (kk == kb) {
        c = o - kb * size + 1;
      } else {
        const KeyT* run = task + rs;
        int64_t lo = 0, hi = re - rs;
        if (kk < kb) {
          while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (!cmp(v, Codec::enc(run[mid]))) lo = mid + 1; else hi = mid;
          }
        } else {
          while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (cmp(Codec::enc(run[mid]), v)) lo = mid + 1; else hi = mid;
          }
        }
        c = lo;
      }
    }
    out[q * k + kk] = c;
  }
}

}  // namespace gms
