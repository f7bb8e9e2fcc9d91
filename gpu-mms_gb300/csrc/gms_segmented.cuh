// Batched (segmented) sort: many independent arrays of uneven length in one
// sort.
//
// No counterpart in the reference, which sorts one array per call
// (GPU-MMS src/multimergesort.hxx:56-141); a batch there is a loop of calls.
//
// For 32-bit keys, segment s of the concatenated input becomes the 64-bit
// composite (s << 32) | ordered_bits(key).  Sorting the composites ascending
// orders by segment first, so every segment's keys stay inside the segment's
// own range and come out sorted: one 64-bit sort of the whole batch (each
// round one launch over all segments) sorts every segment.  Keys are then
// restored from the low 32 bits.
#pragma once

#include <cstdint>

#include "gms_device.cuh"

namespace gms {

// Elements per CTA of the composite build: the CTA finds the segments that
// overlap its chunk once, then each thread finds its element's segment among
// them (a short search in shared memory).
constexpr int kSegChunk = 4096;
constexpr int kSegThreads = 256;
constexpr int kSegMaxLocal = 1024;  // segments cached per chunk; more fall back to a global search

template <class Codec32>
__global__ void __launch_bounds__(kSegThreads)
    build_composite_kernel(const uint32_t* __restrict__ keys, const int64_t* __restrict__ off, int64_t nseg,
                           int64_t n, uint64_t* __restrict__ comp) {
  __shared__ int64_t s_off[kSegMaxLocal + 1];
  __shared__ int64_t s_first;
  __shared__ int s_cnt;
  const int64_t c0 = (int64_t)blockIdx.x * kSegChunk;
  if (c0 >= n) return;
  const int64_t c1 = c0 + kSegChunk < n ? c0 + kSegChunk : n;
  if (threadIdx.x == 0) {
    // first segment s with off[s+1] > c0 (segments may be empty)
    int64_t lo = 0, hi = nseg - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (off[mid + 1] > c0) hi = mid; else lo = mid + 1;
    }
    s_first = lo;
    // segments overlapping [c0, c1): s_first .. last with off[s] < c1
    int64_t lo2 = lo, hi2 = nseg - 1;
    while (lo2 < hi2) {
      const int64_t mid = (lo2 + hi2 + 1) >> 1;
      if (off[mid] < c1) lo2 = mid; else hi2 = mid - 1;
    }
    const int64_t cnt = lo2 - lo + 1;
    s_cnt = cnt > kSegMaxLocal ? -1 : (int)cnt;
  }
  __syncthreads();
  const int cnt = s_cnt;
  const int64_t first = s_first;
  if (cnt > 0) {
    for (int i = threadIdx.x; i <= cnt; i += blockDim.x) s_off[i] = off[first + i];
  }
  __syncthreads();
  for (int64_t p = c0 + threadIdx.x; p < c1; p += blockDim.x) {
    int64_t seg;
    if (cnt > 0) {
      int lo = 0, hi = cnt - 1;  // last local segment whose start <= p
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_off[mid] <= p) lo = mid; else hi = mid - 1;
      }
      seg = first + lo;
    } else {
      int64_t lo = first, hi = nseg - 1;
      while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= p) lo = mid; else hi = mid - 1;
      }
      seg = lo;
    }
    comp[p] = ((uint64_t)seg << 32) | (uint64_t)Codec32::enc(keys[p]);
  }
}

template <class Codec32>
__global__ void extract_composite_kernel(const uint64_t* __restrict__ comp, uint32_t* __restrict__ out, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    out[p] = Codec32::dec((uint32_t)comp[p]);
  }
}

}  // namespace gms
