// GPU library baselines for the int32 sort workload (not part of the library).
//
// The reference ships a thrust comparison program (GPU-MMS src/thrust.cu:32-68)
// that times thrust::sort with a user comparator.  This program times, on the
// same kind of input as the bench (n int32 keys uniform in [0, 2^31-1)):
//   radix  thrust::sort(keys)               (thrust dispatches to CUB's radix sort)
//   merge  thrust::sort(keys, less functor) (a user comparator: CUB's merge sort,
//          a comparison sort like this library's)
// The reference's comparator `a*a+1 <= b*b+3` is not a strict weak order, so
// plain `<` is used.  Each repetition sorts a fresh device copy of the input;
// CUDA events bracket the sort only (thrust's own temporary allocation
// included, as it ships).  Prints one JSON line.
//
// Usage: thrust_baseline <n> [reps] [kv64]
//   kv64: uint64 keys with an int32 payload, stable_sort_by_key instead
#include <thrust/copy.h>
#include <thrust/device_vector.h>
#include <thrust/equal.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct Less {
  __host__ __device__ bool operator()(int32_t a, int32_t b) const { return a < b; }
};

__global__ void fill_uniform(int32_t* a, int64_t n, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t x = seed ^ (uint64_t)i;  // splitmix64
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    a[i] = (int32_t)((x >> 33) % 2147483647ull);
  }
}

template <class F>
static double median_ms(int reps, thrust::device_vector<int32_t>& src, thrust::device_vector<int32_t>& work, F sort) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  std::vector<float> t;
  for (int r = 0; r < reps + 1; ++r) {  // the first run warms up
    thrust::copy(src.begin(), src.end(), work.begin());
    cudaDeviceSynchronize();
    cudaEventRecord(a);
    sort();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (r) t.push_back(ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  std::sort(t.begin(), t.end());
  return t[t.size() / 2];
}

struct Less64 {
  __host__ __device__ bool operator()(uint64_t a, uint64_t b) const { return a < b; }
};

__global__ void fill_u64(uint64_t* k, int32_t* v, int64_t n, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t x = seed ^ (uint64_t)i;  // splitmix64
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    k[i] = x ^ (x >> 31);
    v[i] = (int32_t)i;
  }
}

// uint64 keys + int32 payload, stable: thrust::stable_sort_by_key with the
// default order (CUB radix sort) and with a comparator (CUB merge sort).
static int run_kv64(int64_t n, int reps) {
  thrust::device_vector<uint64_t> ksrc(n), k(n);
  thrust::device_vector<int32_t> vsrc(n), v(n), vradix(n);
  fill_u64<<<1024, 256>>>(thrust::raw_pointer_cast(ksrc.data()), thrust::raw_pointer_cast(vsrc.data()), n, 1);
  cudaDeviceSynchronize();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto time = [&](auto sort) {
    std::vector<float> t;
    for (int r = 0; r < reps + 1; ++r) {
      thrust::copy(ksrc.begin(), ksrc.end(), k.begin());
      thrust::copy(vsrc.begin(), vsrc.end(), v.begin());
      cudaDeviceSynchronize();
      cudaEventRecord(a);
      sort();
      cudaEventRecord(b);
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (r) t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    return (double)t[t.size() / 2];
  };
  const double radix_ms = time([&] { thrust::stable_sort_by_key(thrust::device, k.begin(), k.end(), v.begin()); });
  thrust::copy(v.begin(), v.end(), vradix.begin());
  const double merge_ms =
      time([&] { thrust::stable_sort_by_key(thrust::device, k.begin(), k.end(), v.begin(), Less64()); });
  const bool same = thrust::equal(v.begin(), v.end(), vradix.begin());
  const cudaError_t e = cudaGetLastError();
  printf("{\"n\": %lld, \"reps\": %d, \"kv64_radix_ms\": %.4f, \"kv64_radix_gkeys_s\": %.3f, "
         "\"kv64_merge_ms\": %.4f, \"kv64_merge_gkeys_s\": %.3f, \"agree\": %s, \"cuda\": \"%s\"}\n",
         (long long)n, reps, radix_ms, n / radix_ms / 1e6, merge_ms, n / merge_ms / 1e6, same ? "true" : "false",
         cudaGetErrorName(e));
  return (same && e == cudaSuccess) ? 0 : 1;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <n> [reps]\n", argv[0]);
    return 2;
  }
  const int64_t n = atoll(argv[1]);
  const int reps = argc > 2 ? atoi(argv[2]) : 5;
  if (n <= 0 || reps <= 0) {
    fprintf(stderr, "n and reps must be positive\n");
    return 2;
  }
  if (argc > 3 && strcmp(argv[3], "kv64") == 0) return run_kv64(n, reps);
  thrust::device_vector<int32_t> src(n), work(n), radix_out(n);
  fill_uniform<<<1024, 256>>>(thrust::raw_pointer_cast(src.data()), n, 1);
  cudaDeviceSynchronize();
  const double radix_ms = median_ms(reps, src, work, [&] { thrust::sort(thrust::device, work.begin(), work.end()); });
  thrust::copy(work.begin(), work.end(), radix_out.begin());
  const double merge_ms =
      median_ms(reps, src, work, [&] { thrust::sort(thrust::device, work.begin(), work.end(), Less()); });
  const bool same = thrust::equal(work.begin(), work.end(), radix_out.begin());
  const bool sorted = thrust::is_sorted(thrust::device, work.begin(), work.end());
  const cudaError_t e = cudaGetLastError();
  printf("{\"n\": %lld, \"reps\": %d, \"radix_ms\": %.4f, \"radix_gkeys_s\": %.3f, \"merge_ms\": %.4f, "
         "\"merge_gkeys_s\": %.3f, \"agree\": %s, \"cuda\": \"%s\"}\n",
         (long long)n, reps, radix_ms, n / radix_ms / 1e6, merge_ms, n / merge_ms / 1e6,
         (same && sorted) ? "true" : "false", cudaGetErrorName(e));
  return (same && sorted && e == cudaSuccess) ? 0 : 1;
}
