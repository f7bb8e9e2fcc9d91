// Bulk-copy (TMA) staging for the K-way merge round on sm_103a.
//
// Reference counterpart: the list-head refill of the minBlockHeap,
// fillEmptyLeaf / buildHeap (GPU-MMS src/io-merge-gen.hxx:137-145, 273-303),
// which loads 32-key blocks with ordinary per-thread loads while the heap
// waits.  Here one lane per run issues a single cp.async.bulk for its whole
// segment of the next tile; completion is tracked by an mbarrier transaction
// count, so the copy of tile i+1 runs while tile i is being merged.
#pragma once

#include <cstdint>

#include "gms_device.cuh"

namespace gms {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before its
// later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy; dst/src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// 16-byte asynchronous global -> shared copy (cp.async, bypassing L1);
// completion is waited for by group (cp_async_wait_all).  Both addresses must
// be 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait.  Returns false if the phase did not complete within the limit
// (the caller reports it and stops; nothing spins forever).
//
// After a timeout the kernels set DEV_COPY_TIMEOUT, wait once more (bounded)
// so that copies still in flight can land, and then leave the CTA.  If that
// second wait also runs out, the CTA exits with bulk copies possibly still
// writing its shared memory, which the PTX memory model leaves undefined;
// this exit is accepted only because the status bit has already marked the
// whole result invalid, and the only other choice would be to spin without a
// bound.  A CTA that timed out issues no further copies.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

// Placement of one run segment [A, E) (bytes) in a staging buffer: the
// segment's 16-byte-aligned superset [a16, e16) is reserved; the part of it
// inside the array's own 16-byte-aligned interior is bulk-copied, and the few
// bytes at the array's unaligned ends (never more than 15 per end) are loaded
// with plain loads.
struct SegCopy {
  uint64_t a16, e16;  // reserved superset (global byte addresses)
  uint64_t bs, be;    // bulk-copied part (be <= bs: none)
};

__device__ __forceinline__ SegCopy seg_copy(uint64_t A, uint64_t E, uint64_t arr_lo, uint64_t arr_hi) {
  SegCopy c;
  c.a16 = A & ~15ull;
  c.e16 = (E + 15) & ~15ull;
  const uint64_t lo16 = (arr_lo + 15) & ~15ull;
  const uint64_t hi16 = arr_hi & ~15ull;
  c.bs = c.a16 > lo16 ? c.a16 : lo16;
  c.be = c.e16 < hi16 ? c.e16 : hi16;
  if (E <= A) {
    c.a16 = c.e16 = c.bs = c.be = A & ~15ull;
  }
  return c;
}

}  // namespace gms
