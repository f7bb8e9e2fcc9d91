// CPU oracle for the multiway mergesort hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, the
// drop-in header, the Python binding) links or calls this file.  It is loaded
// by the tests (as the parity checker), by __graft_entry__.smoke() (as the
// checker) and by bench.py (the CPU baseline leg and the `--impl reference`
// arm), and nowhere else.
//
// What it restates, with the reference file:line each function follows
// (paths are relative to the GPU-MMS source tree):
//
//  * gmo_sort_*            -- the result contract of multimergesort<T,cmp>
//                             (src/multimergesort.hxx:56-141): the array sorted
//                             ascending under the plugin comparator cmp<T>
//                             (src/cmp.hxx:37-46, default `a < b`).  For a
//                             strict weak order whose equivalent keys are
//                             bit-identical the sorted output is unique, so
//                             std::sort is bit-identical to any correct sort.
//  * gmo_tile_sort_*       -- squareSort (src/basecase/squareSort.hxx:62-131):
//                             every M-element tile sorted in place, plus the
//                             N%M tail sorted (squareSort.hxx:69-87).
//  * gmo_merge_level_*     -- one merge round of the host loop
//                             (src/multimergesort.hxx:87-135 + multimergeLevel
//                             155-209): every group of K sorted runs of length
//                             `size` merged into one run; the edge group may be
//                             short (edgeCaseTaskSize, multimergesort.hxx:90).
//  * gmo_find_partitions_* -- findPartitions (src/warp-partition.hxx:488-532):
//                             for a target output rank of a K-way merge task,
//                             the number of elements each input list
//                             contributes.  Ties are broken by list index (the
//                             stable order), which is the order the merged
//                             output must have.
//  * gmo_ref_random_list   -- create_random_list (src/buildData.h:54-65) after
//                             srand(seed) (src/testMM.cu:156): keys rand()%RANGE
//                             with RANGE=1024 (src/params.h:35), two rand()
//                             calls per element, the second only feeding the
//                             upper half of a 64-bit DATATYPE.
//  * gmo_selection_sort_i32 -- selection_sort<T,host_cmp>
//                             (src/testMM.cu:308-320), the reference's own CPU
//                             checker for the base case.
//
// Key/value sorts follow std::stable_sort ordered by key, which is the order
// (key, original index).  Floating-point keys are ordered by IEEE-754
// totalOrder over their bit patterns (-NaN < -Inf < ... < -0 < +0 < ... <
// +Inf < +NaN).
//
// The synthetic generators (gmo_gen_*) produce the seeded input families the
// benchmarks and parity tests use; they draw from std::mt19937_64 only and map
// the raw 64-bit words themselves, so x86-64 and aarch64 produce identical
// arrays.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <thread>
#include <vector>
#ifdef _OPENMP
#include <parallel/algorithm>
#include <omp.h>
#endif

namespace {

inline uint32_t f32_order(uint32_t b) { return (b & 0x80000000u) ? ~b : (b | 0x80000000u); }
inline uint64_t f64_order(uint64_t b) {
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

struct F32Less {
  bool operator()(float a, float b) const {
    uint32_t x, y;
    std::memcpy(&x, &a, 4);
    std::memcpy(&y, &b, 4);
    return f32_order(x) < f32_order(y);
  }
};
struct F64Less {
  bool operator()(double a, double b) const {
    uint64_t x, y;
    std::memcpy(&x, &a, 8);
    std::memcpy(&y, &b, 8);
    return f64_order(x) < f64_order(y);
  }
};

template <class T, class C>
void kv_stable(T* keys, int32_t* vals, int64_t n, C less) {
  std::vector<std::pair<T, int32_t>> v((size_t)n);
  for (int64_t i = 0; i < n; ++i) v[i] = {keys[i], vals[i]};
  std::stable_sort(v.begin(), v.end(),
                   [&](const std::pair<T, int32_t>& a, const std::pair<T, int32_t>& b) {
                     return less(a.first, b.first);
                   });
  for (int64_t i = 0; i < n; ++i) {
    keys[i] = v[i].first;
    vals[i] = v[i].second;
  }
}

// Merge groups of K runs of length L (stable: run order, then position).
template <class T, class C>
void merge_level(const T* in, T* out, int64_t n, int64_t L, int K, C less) {
  const int64_t task = L * (int64_t)K;
  for (int64_t g = 0; g < n; g += task) {
    const int64_t e = std::min(n, g + task);
    std::copy(in + g, in + e, out + g);
    // cascade of stable in-place merges keeps the (run, position) order
    for (int64_t w = L; w < e - g; w *= 2) {
      for (int64_t s = g; s + w < e; s += 2 * w) {
        std::inplace_merge(out + s, out + s + w, out + std::min(e, s + 2 * w), less);
      }
    }
  }
}

// Co-ranks of a K-way merge task at target ranks (stable tie-break).
template <class T, class C>
void find_partitions(const T* task, int64_t size, int K, int64_t task_size, const int64_t* ranks,
                     int64_t nranks, int64_t* out, C less) {
  // Merge with run tags, then count tags below each rank.
  std::vector<std::pair<T, int>> v;
  v.reserve((size_t)task_size);
  for (int k = 0; k < K; ++k) {
    const int64_t s = k * size, e = std::min(task_size, (k + 1) * size);
    for (int64_t i = s; i < e; ++i) v.push_back({task[i], k});
  }
  std::stable_sort(v.begin(), v.end(), [&](const std::pair<T, int>& a, const std::pair<T, int>& b) {
    return less(a.first, b.first);
  });
  std::vector<int64_t> cnt((size_t)K, 0);
  std::vector<int64_t> order(nranks);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ranks[a] < ranks[b]; });
  int64_t pos = 0;
  for (int64_t oi = 0; oi < nranks; ++oi) {
    const int64_t q = order[oi];
    const int64_t r = std::min<int64_t>(std::max<int64_t>(ranks[q], 0), task_size);
    while (pos < r) cnt[v[pos++].second]++;
    for (int k = 0; k < K; ++k) out[q * K + k] = cnt[k];
  }
}

inline double u01(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" {

int gmo_version() { return 1; }

// ---- plain sorts (multimergesort result contract) -------------------------
void gmo_sort_i32(int32_t* a, int64_t n) { std::sort(a, a + n); }
void gmo_sort_u32(uint32_t* a, int64_t n) { std::sort(a, a + n); }
void gmo_sort_i64(int64_t* a, int64_t n) { std::sort(a, a + n); }
void gmo_sort_u64(uint64_t* a, int64_t n) { std::sort(a, a + n); }
void gmo_sort_f32(float* a, int64_t n) { std::sort(a, a + n, F32Less()); }
void gmo_sort_f64(double* a, int64_t n) { std::sort(a, a + n, F64Less()); }

// Multithreaded std::sort (libstdc++ parallel mode) -- CPU baseline only.
double gmo_par_sort_i32(int32_t* a, int64_t n, int threads) {
#ifdef _OPENMP
  if (threads > 1) {
    omp_set_num_threads(threads);
    __gnu_parallel::sort(a, a + n);
    return (double)threads;
  }
#endif
  std::sort(a, a + n);
  return 1.0;
}
int gmo_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// ---- key/value: std::stable_sort by key == order (key, original index) ---
void gmo_sort_kv_u32_i32(uint32_t* k, int32_t* v, int64_t n) { kv_stable(k, v, n, std::less<uint32_t>()); }
void gmo_sort_kv_i32_i32(int32_t* k, int32_t* v, int64_t n) { kv_stable(k, v, n, std::less<int32_t>()); }
void gmo_sort_kv_u64_i32(uint64_t* k, int32_t* v, int64_t n) { kv_stable(k, v, n, std::less<uint64_t>()); }
void gmo_sort_kv_i64_i32(int64_t* k, int32_t* v, int64_t n) { kv_stable(k, v, n, std::less<int64_t>()); }
void gmo_sort_kv_f32_i32(float* k, int32_t* v, int64_t n) { kv_stable(k, v, n, F32Less()); }
void gmo_sort_kv_f64_i32(double* k, int32_t* v, int64_t n) { kv_stable(k, v, n, F64Less()); }

// ---- segmented: each [off[s], off[s+1]) sorted independently -------------
void gmo_segmented_sort_i32(int32_t* a, const int64_t* off, int64_t nseg) {
  for (int64_t s = 0; s < nseg; ++s) std::sort(a + off[s], a + off[s + 1]);
}
void gmo_segmented_sort_u64(uint64_t* a, const int64_t* off, int64_t nseg) {
  for (int64_t s = 0; s < nseg; ++s) std::sort(a + off[s], a + off[s + 1]);
}
void gmo_segmented_sort_kv_u64_i32(uint64_t* k, int32_t* v, const int64_t* off, int64_t nseg) {
  for (int64_t s = 0; s < nseg; ++s) kv_stable(k + off[s], v + off[s], off[s + 1] - off[s], std::less<uint64_t>());
}

// ---- base case: squareSort contract ---------------------------------------
void gmo_tile_sort_i32(int32_t* a, int64_t n, int64_t tile) {
  for (int64_t s = 0; s < n; s += tile) std::sort(a + s, a + std::min(n, s + tile));
}
void gmo_tile_sort_u64(uint64_t* a, int64_t n, int64_t tile) {
  for (int64_t s = 0; s < n; s += tile) std::sort(a + s, a + std::min(n, s + tile));
}

// ---- one merge round: groups of K runs of length L ------------------------
void gmo_merge_level_i32(const int32_t* in, int32_t* out, int64_t n, int64_t L, int K) {
  merge_level(in, out, n, L, K, std::less<int32_t>());
}
void gmo_merge_level_u64(const uint64_t* in, uint64_t* out, int64_t n, int64_t L, int K) {
  merge_level(in, out, n, L, K, std::less<uint64_t>());
}

// ---- splitter: co-ranks of one K-way task at given output ranks ------------
void gmo_find_partitions_i32(const int32_t* task, int64_t size, int K, int64_t task_size,
                             const int64_t* ranks, int64_t nranks, int64_t* out) {
  find_partitions(task, size, K, task_size, ranks, nranks, out, std::less<int32_t>());
}

// ---- the reference's own test input and CPU checker ------------------------
void gmo_ref_random_list(int32_t* data, int64_t n, unsigned seed) {
  srand(seed);
  for (int64_t i = 0; i < n; ++i) {
    const int v = rand() % 1024;
    (void)rand();  // second draw only reaches the upper half of a 64-bit key
    data[i] = v;
  }
}
void gmo_selection_sort_i32(int32_t* a, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t j = i + 1; j < n; ++j) {
      if (a[j] < a[i]) std::swap(a[i], a[j]);
    }
  }
}

// ---- seeded synthetic inputs ------------------------------------------------
// dist: 0 uniform [0, 2^31-1); 1 sorted; 2 reverse sorted; 3 all-equal (42);
//       4 sixteen distinct values drawn uniformly; 5 Zipf s=1.2 over 2^20 ranks
//       (value = rank-1); 6 uniform over the full int32 range (negatives too).
void gmo_gen_i32(int32_t* a, int64_t n, int dist, uint64_t seed) {
  std::mt19937_64 g(seed);
  switch (dist) {
    case 0:
      for (int64_t i = 0; i < n; ++i) a[i] = (int32_t)(g() % 2147483647ull);
      break;
    case 1:
    case 2: {
      for (int64_t i = 0; i < n; ++i) a[i] = (int32_t)(g() % 2147483647ull);
      std::sort(a, a + n);
      if (dist == 2) std::reverse(a, a + n);
      break;
    }
    case 3:
      for (int64_t i = 0; i < n; ++i) a[i] = 42;
      break;
    case 4: {
      int32_t vals[16];
      for (int i = 0; i < 16; ++i) vals[i] = (int32_t)(g() % 2147483647ull);
      for (int64_t i = 0; i < n; ++i) a[i] = vals[g() & 15];
      break;
    }
    case 5: {
      const int R = 1 << 20;
      std::vector<double> cdf(R);
      double acc = 0;
      for (int r = 0; r < R; ++r) {
        acc += std::pow((double)(r + 1), -1.2);
        cdf[r] = acc;
      }
      for (int r = 0; r < R; ++r) cdf[r] /= acc;
      for (int64_t i = 0; i < n; ++i) {
        const double u = u01(g);
        int64_t r = std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin();
        if (r >= R) r = R - 1;
        a[i] = (int32_t)r;
      }
      break;
    }
    default:
      for (int64_t i = 0; i < n; ++i) a[i] = (int32_t)(uint32_t)g();
      break;
  }
}
void gmo_gen_u64(uint64_t* a, int64_t n, uint64_t seed) {
  std::mt19937_64 g(seed);
  for (int64_t i = 0; i < n; ++i) a[i] = g();
}
// Standard normal float32, then 1% replaced by +-0.0 (half each) and 0.1% by NaN
// (sign and payload drawn too, so the total order over NaNs is exercised).
void gmo_gen_f32(float* a, int64_t n, uint64_t seed) {
  std::mt19937_64 g(seed);
  for (int64_t i = 0; i < n; i += 2) {
    double u1 = u01(g), u2 = u01(g);
    if (u1 < 1e-300) u1 = 1e-300;
    const double r = std::sqrt(-2.0 * std::log(u1));
    a[i] = (float)(r * std::cos(6.283185307179586 * u2));
    if (i + 1 < n) a[i + 1] = (float)(r * std::sin(6.283185307179586 * u2));
  }
  for (int64_t i = 0; i < n; ++i) {
    const uint64_t w = g();
    const uint32_t sel = (uint32_t)(w % 100000ull);
    if (sel < 1000) {
      a[i] = (sel & 1) ? -0.0f : 0.0f;
    } else if (sel < 1100) {
      uint32_t bits = 0x7fc00000u | (uint32_t)((w >> 20) & 0x3fffffu);
      if ((w >> 50) & 1) bits |= 0x80000000u;
      std::memcpy(&a[i], &bits, 4);
    }
  }
}
// Segment lengths log-uniform in [lo, hi]; returns the total length.
int64_t gmo_gen_seg_lengths(int64_t* len, int64_t nseg, int64_t lo, int64_t hi, uint64_t seed) {
  std::mt19937_64 g(seed);
  const double a = std::log((double)lo), b = std::log((double)hi + 1.0);
  int64_t tot = 0;
  for (int64_t s = 0; s < nseg; ++s) {
    int64_t v = (int64_t)std::floor(std::exp(a + (b - a) * u01(g)));
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    len[s] = v;
    tot += v;
  }
  return tot;
}

// ---- checkers ---------------------------------------------------------------
// Index of the first position where a and b differ, or -1.
int64_t gmo_first_diff(const void* a, const void* b, int64_t n, int elem_bytes) {
  const unsigned char* x = (const unsigned char*)a;
  const unsigned char* y = (const unsigned char*)b;
  for (int64_t i = 0; i < n; ++i) {
    if (std::memcmp(x + i * elem_bytes, y + i * elem_bytes, (size_t)elem_bytes) != 0) return i;
  }
  return -1;
}

}  // extern "C"
