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
 * work, calls from several host threads at once are safe, and errors return
 * nullptr (message on stderr and in gms_dropin_last_error()).  threadBlocks is
 * accepted as a hint; the grids are sized by the data.
 *
 * Built-in 32- and 64-bit integer keys under the default cmp<T> take the same
 * keys-only engine as the library's gms_sort_i32 / _u32 / _i64 / _u64 (warp
 * base case, bulk-copied merge tiles; equal integers are identical, so the
 * result is that of a stable sort).  Every other type or comparator takes the
 * generic stable engine, which inlines the comparator into its kernels.
 */
#ifndef GMS_MULTIMERGESORT_HXX_
#define GMS_MULTIMERGESORT_HXX_

#include <cstdio>
#include <vector>
#include <cuda_runtime.h>

#include "params.h"
#include "cmp.hxx"
#include "../gpu-mms_gb300/csrc/gms_engines.cuh"
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

// True when (T, f) sorts through the library's keys-only engine: a built-in
// 32/64-bit integer and the default comparator cmp<T> of cmp.hxx.
template <typename T, int (*f)(T, T)>
constexpr bool fast_keys() {
#ifndef GMS_USER_CMP
  if constexpr (gms_engines::BuiltinKey<T>::value) {
    return f == &cmp<T>;
  }
#endif
  return false;
}

inline const char*& last_error_slot() {
  static thread_local const char* msg = "";
  return msg;
}

// Device scratch of the calling host thread, one grow-only buffer per device,
// so concurrent calls from several threads never share a buffer.  A call is
// synchronous, so when a buffer is regrown no earlier call of this thread
// still uses it.  Buffers are freed when the thread exits.
struct ThreadScratch {
  struct Slot {
    int dev;
    void* ptr;
    size_t have;
  };
  std::vector<Slot> slots;
  ~ThreadScratch() {
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return;
    for (Slot& s : slots) {
      if (cudaSetDevice(s.dev) == cudaSuccess) cudaFree(s.ptr);
    }
    cudaSetDevice(cur);
  }
};

inline void* scratch(size_t bytes, cudaError_t* err) {
  static thread_local ThreadScratch ts;
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess) return nullptr;
  ThreadScratch::Slot* slot = nullptr;
  for (ThreadScratch::Slot& s : ts.slots) {
    if (s.dev == dev) slot = &s;
  }
  if (!slot) {
    ts.slots.push_back(ThreadScratch::Slot{dev, nullptr, 0});
    slot = &ts.slots.back();
  }
  if (bytes <= slot->have) return slot->ptr;
  if (slot->ptr) {
    cudaFree(slot->ptr);
    slot->ptr = nullptr;
    slot->have = 0;
  }
  *err = cudaMalloc(&slot->ptr, bytes);
  if (*err != cudaSuccess) {
    slot->ptr = nullptr;
    return nullptr;
  }
  slot->have = bytes;
  return slot->ptr;
}

// One sort through engine Eng on keys of stored type KT.  BY_SIZE: the
// fan-in and sample block follow N (gms_engines::balanced_fan_in), as in the
// prebuilt library, unless the caller fixed GMS_K / GMS_SAMPLE_B.
template <class Eng, class KT, bool BY_SIZE = false>
cudaError_t sort_with(KT* input, KT* output, int N) {
  gms::Tune t;
  t.k = GMS_K;
  t.sample_b = GMS_SAMPLE_B;
  if constexpr (BY_SIZE) t = gms_engines::balanced_fan_in((int64_t)N, Eng::BASE_TILE, t);
  const gms::WsLayout l = Eng::plan((int64_t)N, t);
  if (!l.ok) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  void* ws = scratch(gms::ws_bytes_for<KT>(l, t.k), &e);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ws, 0, 256, 0);  // the status word starts clear
  if (e != cudaSuccess) return e;
  const gms::WsPtrs<KT> w = gms::ws_carve<KT>(l, t.k, ws);
  e = Eng::sort(w, input, nullptr, output, nullptr, (int64_t)N, t, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e;
}

template <typename T, int (*f)(T, T)>
T* run(T* input, T* output, int N) {
  static_assert(GMS_K >= 2 && GMS_K <= 32, "GMS_K (fan-in) must be in [2, 32]");
  static_assert(GMS_SAMPLE_B >= 8 && DropinEngine<T, f>::CAPW / GMS_SAMPLE_B - GMS_K >= 1,
                "GMS_SAMPLE_B must be >= 8 and leave room for a merge tile");
  if (N < 0 || (N > 0 && (!input || !output))) {
    last_error_slot() = "multimergesort: bad arguments";
    fprintf(stderr, "%s\n", last_error_slot());
    return nullptr;
  }
  if (N == 0) return output;
  cudaError_t e;
  if constexpr (fast_keys<T, f>()) {
    using BK = gms_engines::BuiltinKey<T>;
    using KT = typename BK::Stored;
#ifdef GMS_FAN_IN_BY_SIZE
    constexpr bool by_size = true;
#else
    constexpr bool by_size = false;
#endif
    e = sort_with<gms_engines::KeysEngine<KT, typename BK::Codec>, KT, by_size>(reinterpret_cast<KT*>(input),
                                                                               reinterpret_cast<KT*>(output), N);
  } else {
    e = sort_with<DropinEngine<T, f>, T>(input, output, N);
  }
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
