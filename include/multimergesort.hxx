/*
 * multimergesort.hxx -- drop-in replacement for GPU-MMS's multimergesort.
 *
 * Header-only, compiled into the caller's translation unit by nvcc for
 * sm_103a, so the caller's comparator is inlined into the kernels:
 *
 *   d_out = multimergesort<T, cmp>(d_in, d_out, h_data, N);              // 4 args
 *   d_out = multimergesort<T, cmp>(d_in, d_out, h_data, threadBlocks, N); // 5 args
 *
 * Replaces: template<typename T, fptr_t f> T* multimergesort(T* input,
 *   T* output, T* h_data, int N)  (src/multimergesort.hxx:56-141) and the
 *   documented 5-argument form (README.md:16-25).
 *
 * Contract (same as the reference): `input` and `output` are device arrays of
 * N elements; `input` is clobbered; the return value points at the buffer that
 * holds the sorted result (always `output` here); `h_data` is unused; the call
 * is synchronous (cudaDeviceSynchronize at the end).  Differences: the result
 * is stable (equivalent elements keep their input order), every key value is
 * valid (no MAXVAL sentinel), N < 1024 works, several T per translation unit
 * work, and errors return nullptr (message on stderr and in
 * gms_dropin_last_error()).  threadBlocks is accepted as a hint; the grids are
 * sized by the data.
 */
#ifndef GMS_MULTIMERGESORT_HXX_
#define GMS_MULTIMERGESORT_HXX_

#include <cstdio>
#include <cuda_runtime.h>

#include "params.h"
#include "cmp.hxx"
#include "../gpu-mms_gb300/csrc/gms_sort.cuh"

namespace gms_dropin {

template <typename T, int (*f)(T, T)>
struct FnLess {
  __device__ __forceinline__ bool operator()(const T& a, const T& b) const { return f(a, b) != 0; }
};

// 256 threads x 17 elements: tiles of 4352 elements, modest shared memory for
// wide user types.
template <typename T, int (*f)(T, T)>
using DropinEngine = gms::Engine<T, gms::NoVal, FnLess<T, f>, gms::IdentityCodec<T>, true, 256, 17>;

inline const char*& last_error_slot() {
  static thread_local const char* msg = "";
  return msg;
}

// Grow-only device scratch shared by every drop-in call of the process.
inline void* scratch(size_t bytes, cudaError_t* err) {
  static void* ptr = nullptr;
  static size_t have = 0;
  *err = cudaSuccess;
  if (bytes <= have) return ptr;
  if (ptr) {
    cudaDeviceSynchronize();
    cudaFree(ptr);
    ptr = nullptr;
    have = 0;
  }
  *err = cudaMalloc(&ptr, bytes);
  if (*err != cudaSuccess) {
    ptr = nullptr;
    return nullptr;
  }
  cudaMemset(ptr, 0, 256);
  have = bytes;
  return ptr;
}

template <typename T, int (*f)(T, T)>
T* run(T* input, T* output, int N) {
  using Eng = DropinEngine<T, f>;
  static_assert(GMS_K >= 2 && GMS_K <= 32, "GMS_K (fan-in) must be in [2, 32]");
  static_assert(GMS_SAMPLE_B >= 8 && Eng::CAPW / GMS_SAMPLE_B - GMS_K >= 1,
                "GMS_SAMPLE_B must be >= 8 and leave room for a merge tile");
  if (N < 0 || (N > 0 && (!input || !output))) {
    last_error_slot() = "multimergesort: bad arguments";
    fprintf(stderr, "%s\n", last_error_slot());
    return nullptr;
  }
  if (N == 0) return output;
  gms::Tune t;
  t.k = GMS_K;
  t.sample_b = GMS_SAMPLE_B;
  const gms::WsLayout l = Eng::plan((int64_t)N, t);
  cudaError_t e = cudaSuccess;
  void* ws = scratch(gms::ws_bytes_for<T>(l, t.k), &e);
  if (e == cudaSuccess) {
    const gms::WsPtrs<T> w = gms::ws_carve<T>(l, t.k, ws);
    e = Eng::sort(w, input, nullptr, output, nullptr, (int64_t)N, t, 0);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    last_error_slot() = cudaGetErrorString(e);
    fprintf(stderr, "multimergesort: %s\n", last_error_slot());
    return nullptr;
  }
  return output;
}

}  // namespace gms_dropin

inline const char* gms_dropin_last_error() { return gms_dropin::last_error_slot(); }

// 4-argument form (src/multimergesort.hxx:56-57)
template <typename T, int (*f)(T, T)>
T* multimergesort(T* input, T* output, T* h_data, int N) {
  (void)h_data;
  return gms_dropin::run<T, f>(input, output, N);
}

// 5-argument form (README.md:16-25)
template <typename T, int (*f)(T, T)>
T* multimergesort(T* input, T* output, T* h_data, int threadBlocks, int N) {
  (void)h_data;
  (void)threadBlocks;
  return gms_dropin::run<T, f>(input, output, N);
}

#endif /* GMS_MULTIMERGESORT_HXX_ */
