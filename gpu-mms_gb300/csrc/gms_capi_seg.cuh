// Batched (segmented) sorts through the C ABI: the offsets are read on the
// host, the batch is planned (gms_seg_plan.h: per-segment base tiles and
// merge rounds, groups listed so that none crosses a segment), the plan's
// arrays are uploaded, and the engine runs one launch sequence per round over
// every segment.
//
// No counterpart in the reference, which sorts one array per multimergesort
// call (GPU-MMS src/multimergesort.hxx:56-141).
#pragma once

#include <algorithm>
#include <vector>

#include "gms_capi.cuh"

namespace gms_capi {

// Copies the nseg + 1 offsets to the host (waiting for `st`) and checks
// 0 = off[0] <= off[1] <= ... <= off[nseg] = n.
int read_offsets(const int64_t* off, int64_t nseg, int64_t n, cudaStream_t st, std::vector<int64_t>* h);

// A planned batch: the host plan, the byte layout of its device arrays, the
// bound device view (after seg_upload) and the scratch it needs.
struct SegJob {
  gms::SegPlanH plan;
  gms::SegBlob blob;
  gms::SegDev dev;
  size_t ws_bytes = 0;
};

template <class Eng, class K>
int seg_prepare(const std::vector<int64_t>& off, int64_t nseg, const gms::Tune& t, SegJob* job) {
  job->plan = gms::seg_plan(off.data(), nseg, Eng::seg_geom(t));
  if (job->plan.too_long) return set_error(GMS_ERR_TOO_LARGE, "an array of the batch is longer than 2^31 - 1 keys");
  if (!job->plan.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this batch (sample recursion too deep)");
  job->blob = gms::seg_blob_layout(job->plan);
  job->ws_bytes = gms::ws_bytes_for<K>(gms::seg_ws_layout(job->plan), t.k);
  return GMS_OK;
}

// Copies the plan's arrays to `dblob` (job->blob.bytes bytes, device) on `st`
// and binds the device view to them.
int seg_upload(SegJob* job, void* dblob, cudaStream_t st);

// The int32 batch of a CUDA graph (defined with the 32-bit keys engines):
// plans it, and runs it on caller-owned scratch `ws` (job.ws_bytes) and
// scratch array `tmp` of n keys.
int seg_prepare_i32(const std::vector<int64_t>& off, int64_t nseg, const gms::Tune& t, SegJob* job);
cudaError_t seg_sort_i32(const SegJob& job, void* ws, const int32_t* in, int32_t* tmp, int32_t* out, int64_t n,
                         const gms::Tune& t, cudaStream_t st);

// Batches of the sort server, planned from host offsets (defined with the
// engines of their key type): prepare plans the batch; run binds the plan to
// its device copy `dblob` (the caller uploads seg_blob_fill's bytes there on
// `st`) and sorts with scratch from the stream's cache.
int seg_prepare_kv_u64(const std::vector<int64_t>& off, int64_t nseg, const gms::Tune& t, SegJob* job);
int seg_run_i32(SegJob* job, const void* dblob, const int32_t* in, int32_t* out, int64_t n, const gms::Tune& t,
                cudaStream_t st);
int seg_run_kv_u64(SegJob* job, const void* dblob, const uint64_t* kin, const int32_t* vin, uint64_t* kout,
                   int32_t* vout, int64_t n, const gms::Tune& t, cudaStream_t st);

// Runs a planned batch whose arrays are already on the device at `dblob`.
template <class Eng, class K, class V>
int run_planned(SegJob* job, const void* dblob, const K* in, const V* vin, K* out, V* vout, int64_t n,
                const gms::Tune& t, cudaStream_t st) {
  constexpr bool kv = gms::HasVal<V>::value;
  int status = GMS_OK;
  void* ws = cache_get(0, job->ws_bytes, st, &status);
  if (status != GMS_OK) return status;
  K* tmp = (K*)cache_get(30, sizeof(K) * (size_t)n, st, &status);
  if (status != GMS_OK) return status;
  V* vtmp = nullptr;
  if constexpr (kv) {
    vtmp = (V*)cache_get(31, sizeof(V) * (size_t)n, st, &status);
    if (status != GMS_OK) return status;
  }
  gms::seg_bind(job->plan, job->blob, dblob, &job->dev);
  const gms::WsPtrs<K> w = gms::ws_carve<K>(gms::seg_ws_layout(job->plan), t.k, ws);
  const cudaError_t e = Eng::seg_sort(w, job->dev, in, vin, tmp, vtmp, out, vout, n, t, st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "segmented sort");
}

// One batched sort with scratch from the per-stream cache: `in`/`vin` are
// read only, every array of the batch is sorted into the same range of
// `out`/`vout` (payload sorts are stable).
template <class Eng, class K, class V>
int run_segmented(const K* in, const V* vin, K* out, V* vout, int64_t n, const int64_t* off, int64_t nseg,
                  cudaStream_t st, int dtype) {
  clear_error();
  constexpr bool kv = gms::HasVal<V>::value;
  if (n < 0 || nseg < 0) return set_error(GMS_ERR_INVALID, "n < 0 or nseg < 0");
  if (nseg == 0 && n != 0) return set_error(GMS_ERR_INVALID, "no segments for n > 0 keys");
  if (n == 0 || nseg == 0) return GMS_OK;
  if (!in || !out || !off) return set_error(GMS_ERR_INVALID, "null pointer");
  if (kv && (!vin || !vout)) return set_error(GMS_ERR_INVALID, "null value pointer");
  if (n > ((int64_t)1 << 37)) return set_error(GMS_ERR_TOO_LARGE, "n beyond 2^37");
  if (nseg >= ((int64_t)1 << 31)) return set_error(GMS_ERR_TOO_LARGE, "2^31 segments or more");
  std::vector<int64_t> h;
  int status = read_offsets(off, nseg, n, st, &h);
  if (status != GMS_OK) return status;
  int64_t longest = 0;
  for (int64_t s = 0; s < nseg; ++s) longest = std::max(longest, h[(size_t)(s + 1)] - h[(size_t)s]);
  const gms::Tune t = tune_for_batch(dtype, kv ? 1 : 0, n, longest);
  SegJob job;
  status = seg_prepare<Eng, K>(h, nseg, t, &job);
  if (status != GMS_OK) return status;
  void* ws = cache_get(0, job.ws_bytes, st, &status);
  if (status != GMS_OK) return status;
  void* blob = cache_get(32, job.blob.bytes, st, &status);
  if (status != GMS_OK) return status;
  K* tmp = (K*)cache_get(30, sizeof(K) * (size_t)n, st, &status);
  if (status != GMS_OK) return status;
  V* vtmp = nullptr;
  if constexpr (kv) {
    vtmp = (V*)cache_get(31, sizeof(V) * (size_t)n, st, &status);
    if (status != GMS_OK) return status;
  }
  status = seg_upload(&job, blob, st);
  if (status != GMS_OK) return status;
  const gms::WsPtrs<K> w = gms::ws_carve<K>(gms::seg_ws_layout(job.plan), t.k, ws);
  const cudaError_t e = Eng::seg_sort(w, job.dev, in, vin, tmp, vtmp, out, vout, n, t, st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "segmented sort");
}

}  // namespace gms_capi
