// Drop-in check: a caller written for GPU-MMS's multimergesort<T,cmp>
// (README.md:14-25, src/testMM.cu:175) compiled against this repository's
// include/multimergesort.hxx.  Each case sorts on the GPU through the template
// and compares with std::stable_sort under the same comparator on the host
// (the drop-in sort is stable).  Prints one line per case; exit code 0 only if
// every case matches bit for bit.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "multimergesort.hxx"

// user comparators, written the way cmp.hxx defines cmp<T>
__forceinline__ __device__ int desc_cmp(int a, int b) { return a > b; }
__forceinline__ __device__ int abs_cmp(int a, int b) { return (a < 0 ? -a : a) < (b < 0 ? -b : b); }

// a packed key/value record ordered by key only (cmp.hxx:59-73 style)
struct Rec {
  int key;
  int val;
};
__forceinline__ __device__ int rec_cmp(Rec a, Rec b) { return a.key < b.key; }

// A packed 32-bit key + 32-bit value in the shape of the reference's
// commented testType (cmp.hxx:59-73): the cast to and assignments from a
// 64-bit CASTTYPE word that its warp shuffles need.  This library never shuffles
// keys, but such a type must still compile and sort (by key, stably).
struct PackedKV {
  int key;
  int val;
  __forceinline__ __device__ operator long long() const {
    return (long long)(unsigned)key + (long long)((unsigned long long)(unsigned)val << 32);
  }
  __forceinline__ __device__ PackedKV& operator=(const long long& w) {
    key = (int)w;
    val = (int)(w >> 32);
    return *this;
  }
};
__forceinline__ __device__ int packed_cmp(PackedKV a, PackedKV b) { return a.key < b.key; }

// The reference's alternative comparator examples on a 64-bit word
// (cmp.hxx:41-46): the low 32 bits as a signed int ("L1-norm"), and a
// fraction numerator/denominator packed high/low, compared exactly by
// cross-multiplication (denominators positive).
__forceinline__ __device__ int low32_cmp(long long a, long long b) { return (int)a < (int)b; }
__forceinline__ __device__ int frac_cmp(long long a, long long b) {
  return (long long)(int)(a >> 32) * (int)b < (long long)(int)(b >> 32) * (int)a;
}
static bool host_frac_less(long long a, long long b) {
  return (long long)(int)(a >> 32) * (int)b < (long long)(int)(b >> 32) * (int)a;
}

static int failures = 0;

template <class T, int (*f)(T, T), class HostLess>
static void run_case(const char* name, std::vector<T> h, HostLess less, bool five_args) {
  const int n = (int)h.size();
  T *d_in = nullptr, *d_out = nullptr;
  cudaMalloc(&d_in, sizeof(T) * (n > 0 ? n : 1));
  cudaMalloc(&d_out, sizeof(T) * (n > 0 ? n : 1));
  cudaMemcpy(d_in, h.data(), sizeof(T) * n, cudaMemcpyHostToDevice);
  T* res = five_args ? multimergesort<T, f>(d_in, d_out, h.data(), 482, n) : multimergesort<T, f>(d_in, d_out, h.data(), n);
  std::vector<T> got(n);
  bool ok = res != nullptr;
  if (ok) {
    cudaMemcpy(got.data(), res, sizeof(T) * n, cudaMemcpyDeviceToHost);
    std::vector<T> want = h;
    std::stable_sort(want.begin(), want.end(), less);
    ok = n == 0 || std::memcmp(got.data(), want.data(), sizeof(T) * n) == 0;
  }
  printf("%-28s n=%-8d %s\n", name, n, ok ? "OK" : "MISMATCH");
  if (!ok) ++failures;
  cudaFree(d_in);
  cudaFree(d_out);
}

// Several host threads calling multimergesort at the same moment, each on its
// own arrays, three calls each: the built-in fast path (int, long long) and a
// user comparator side by side.  Every result must be bit-exact.
template <class T, int (*f)(T, T), class HostLess>
static bool thread_sorts(std::vector<T> h, HostLess less, std::atomic<int>* go, int reps) {
  const int n = (int)h.size();
  std::vector<T> want = h;
  std::stable_sort(want.begin(), want.end(), less);
  T *d_in = nullptr, *d_out = nullptr;
  if (cudaMalloc(&d_in, sizeof(T) * n) != cudaSuccess || cudaMalloc(&d_out, sizeof(T) * n) != cudaSuccess) return false;
  go->fetch_add(1);
  while (go->load() < 3) {
  }
  bool ok = true;
  std::vector<T> got(n);
  for (int r = 0; r < reps && ok; ++r) {
    cudaMemcpy(d_in, h.data(), sizeof(T) * n, cudaMemcpyHostToDevice);
    T* res = multimergesort<T, f>(d_in, d_out, h.data(), n);
    ok = res != nullptr && cudaMemcpy(got.data(), res, sizeof(T) * n, cudaMemcpyDeviceToHost) == cudaSuccess &&
         std::memcmp(got.data(), want.data(), sizeof(T) * n) == 0;
  }
  cudaFree(d_in);
  cudaFree(d_out);
  return ok;
}

static void concurrent_case(std::mt19937& g) {
  std::vector<int> a((1 << 22) + 5), c(1000003);
  std::vector<long long> b(3000017);
  for (int& x : a) x = (int)g();
  for (long long& x : b) x = (long long)(((unsigned long long)g() << 32) | g());
  for (int& x : c) x = (int)(g() % 2001) - 1000;
  std::atomic<int> go{0};
  bool ok[3] = {false, false, false};
  std::thread t0([&] { ok[0] = thread_sorts<int, cmp<int>>(a, [](int x, int y) { return x < y; }, &go, 3); });
  std::thread t1([&] {
    ok[1] = thread_sorts<long long, cmp<long long>>(b, [](long long x, long long y) { return x < y; }, &go, 3);
  });
  std::thread t2([&] { ok[2] = thread_sorts<int, desc_cmp>(c, [](int x, int y) { return x > y; }, &go, 3); });
  t0.join();
  t1.join();
  t2.join();
  const bool all = ok[0] && ok[1] && ok[2];
  printf("%-28s %s\n", "3 host threads at once", all ? "OK" : "MISMATCH");
  if (!all) ++failures;
}

int main() {
  std::mt19937 g(1234);
  const int sizes[] = {0, 1, 7, 1000, 4352, 4353, 8193, 300001, (1 << 22) + 3, 1 << 24};
  for (int n : sizes) {
    std::vector<int> a(n);
    for (int& x : a) x = (int)(g() % 2001) - 1000;  // many ties
    run_case<int, cmp<int>>("default cmp<int> (4 args)", a, [](int x, int y) { return x < y; }, false);
    run_case<int, cmp<int>>("default cmp<int> (5 args)", a, [](int x, int y) { return x < y; }, true);
    std::vector<unsigned> u(n);
    for (unsigned& x : u) x = (unsigned)g();
    run_case<unsigned, cmp<unsigned>>("default cmp<unsigned>", u, [](unsigned x, unsigned y) { return x < y; }, false);
    std::vector<long long> ll(n);
    for (long long& x : ll) x = (long long)(((unsigned long long)g() << 32) | g());
    run_case<long long, cmp<long long>>("default cmp<long long>", ll, [](long long x, long long y) { return x < y; },
                                        false);
    run_case<int, desc_cmp>("descending", a, [](int x, int y) { return x > y; }, false);
    run_case<int, abs_cmp>("absolute value (stable)", a, [](int x, int y) { return std::abs(x) < std::abs(y); }, false);
    std::vector<Rec> r(n);
    for (int i = 0; i < n; ++i) r[i] = Rec{(int)(g() % 97), i};
    run_case<Rec, rec_cmp>("key/value record (stable)", r, [](const Rec& x, const Rec& y) { return x.key < y.key; },
                           false);
    std::vector<PackedKV> pk(n);
    for (int i = 0; i < n; ++i) pk[i] = PackedKV{(int)(g() % 301) - 150, i};
    run_case<PackedKV, packed_cmp>("packed testType (stable)", pk,
                                   [](const PackedKV& x, const PackedKV& y) { return x.key < y.key; }, true);
    std::vector<long long> w(n);
    for (int i = 0; i < n; ++i) {
      const long long num = (long long)(g() % 2001) - 1000, den = 1 + (long long)(g() % 64);
      w[i] = (long long)((unsigned long long)num << 32) | (unsigned long long)den;
    }
    run_case<long long, frac_cmp>("fraction num/den (stable)", w, host_frac_less, false);
    for (int i = 0; i < n; ++i) w[i] = (long long)(((unsigned long long)g() << 32) | g());
    run_case<long long, low32_cmp>("low 32 bits as int (stable)", w,
                                   [](long long x, long long y) { return (int)x < (int)y; }, false);
  }
  // the full key range: MAXVAL is an ordinary key here
  std::vector<int> ext(100003);
  for (int& x : ext) x = (g() & 1) ? MAXVAL : (int)(g() % 5) - 2;
  run_case<int, cmp<int>>("MAXVAL keys", ext, [](int x, int y) { return x < y; }, false);
  concurrent_case(g);
  printf(failures ? "DROPIN FAILED\n" : "DROPIN OK\n");
  return failures ? 1 : 0;
}
