// C ABI: key/value sorts (stable), int32 payload.
#include "gms_capi.cuh"
#include "gms_capi_seg.cuh"

using namespace gms_capi;

namespace {

template <class Eng, class K>
int kv(void* ki, int32_t* vi, void* ko, int32_t* vo, int64_t n, void* st, int dtype) {
  return run_sort<Eng, K, int32_t>((K*)ki, vi, (K*)ko, vo, n, (cudaStream_t)st, dtype);
}

}  // namespace

int gms_capi::seg_prepare_kv_u64(const std::vector<int64_t>& off, int64_t nseg, const gms::Tune& t, SegJob* job) {
  return seg_prepare<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t>(off, nseg, t, job);
}

int gms_capi::seg_run_kv_u64(SegJob* job, const void* dblob, const uint64_t* kin, const int32_t* vin, uint64_t* kout,
                             int32_t* vout, int64_t n, const gms::Tune& t, cudaStream_t st) {
  return run_planned<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t, int32_t>(job, dblob, kin, vin, kout,
                                                                                        vout, n, t, st);
}

int gms_capi::sort_kv_ws(int dtype, void* ki, int32_t* vi, void* ko, int32_t* vo, int64_t n, void* ws, size_t bytes,
                         cudaStream_t st) {
  uint32_t *i4 = (uint32_t*)ki, *o4 = (uint32_t*)ko;
  uint64_t *i8 = (uint64_t*)ki, *o8 = (uint64_t*)ko;
  switch (dtype) {
    case 0: return run_sort<KvEngine<uint32_t, gms::SignFlip32>, uint32_t, int32_t>(i4, vi, o4, vo, n, st, 0, ws, bytes);
    case 1:
      return run_sort<KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>, uint32_t, int32_t>(i4, vi, o4, vo, n, st, 1, ws,
                                                                                          bytes);
    case 2: return run_sort<KvEngine<uint32_t, gms::FloatOrder32>, uint32_t, int32_t>(i4, vi, o4, vo, n, st, 2, ws, bytes);
    case 3: return run_sort<KvEngine<uint64_t, gms::SignFlip64>, uint64_t, int32_t>(i8, vi, o8, vo, n, st, 3, ws, bytes);
    case 4:
      return run_sort<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t, int32_t>(i8, vi, o8, vo, n, st, 4, ws,
                                                                                          bytes);
    default:
      return run_sort<KvEngine<uint64_t, gms::FloatOrder64>, uint64_t, int32_t>(i8, vi, o8, vo, n, st, 5, ws, bytes);
  }
}

extern "C" {

int gms_sort_kv_i32_i32(int32_t* ki, int32_t* vi, int32_t* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint32_t, gms::SignFlip32>, uint32_t>(ki, vi, ko, vo, n, st, 0);
}
int gms_sort_kv_u32_i32(uint32_t* ki, int32_t* vi, uint32_t* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>, uint32_t>(ki, vi, ko, vo, n, st, 1);
}
int gms_sort_kv_f32_i32(float* ki, int32_t* vi, float* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint32_t, gms::FloatOrder32>, uint32_t>(ki, vi, ko, vo, n, st, 2);
}
int gms_sort_kv_i64_i32(int64_t* ki, int32_t* vi, int64_t* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint64_t, gms::SignFlip64>, uint64_t>(ki, vi, ko, vo, n, st, 3);
}
int gms_sort_kv_u64_i32(uint64_t* ki, int32_t* vi, uint64_t* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t>(ki, vi, ko, vo, n, st, 4);
}
int gms_sort_kv_f64_i32(double* ki, int32_t* vi, double* ko, int32_t* vo, int64_t n, int tb, void* st) {
  (void)tb;
  return kv<KvEngine<uint64_t, gms::FloatOrder64>, uint64_t>(ki, vi, ko, vo, n, st, 5);
}

int gms_sort_host_kv_u64_i32(const uint64_t* keys_in, const int32_t* vals_in, uint64_t* keys_out, int32_t* vals_out,
                             int64_t n, void* stv) {
  clear_error();
  if (n < 0) return set_error(GMS_ERR_INVALID, "n < 0");
  if (n == 0) return GMS_OK;
  if (!keys_in || !vals_in || !keys_out || !vals_out) return set_error(GMS_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stv;
  int status = GMS_OK;
  const size_t kb = sizeof(uint64_t) * (size_t)n, vb = sizeof(int32_t) * (size_t)n;
  void* dki = cache_get(20, kb, st, &status);
  if (status != GMS_OK) return status;
  void* dko = cache_get(21, kb, st, &status);
  if (status != GMS_OK) return status;
  void* dvi = cache_get(22, vb, st, &status);
  if (status != GMS_OK) return status;
  void* dvo = cache_get(23, vb, st, &status);
  if (status != GMS_OK) return status;
  cudaError_t e = cudaMemcpyAsync(dki, keys_in, kb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dvi, vals_in, vb, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync H2D");
  status = kv<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t>(dki, (int32_t*)dvi, dko, (int32_t*)dvo, n,
                                                                         stv, 4);
  if (status != GMS_OK) return status;
  e = cudaMemcpyAsync(keys_out, dko, kb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vals_out, dvo, vb, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync D2H");
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "cudaStreamSynchronize");
}

int gms_segmented_sort_kv_i32_i32(const int32_t* ki, const int32_t* vi, int32_t* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint32_t, gms::SignFlip32>, uint32_t, int32_t>(
      (const uint32_t*)ki, vi, (uint32_t*)ko, vo, n, offsets, nseg, (cudaStream_t)st, 0);
}
int gms_segmented_sort_kv_u32_i32(const uint32_t* ki, const int32_t* vi, uint32_t* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>, uint32_t, int32_t>(
      ki, vi, ko, vo, n, offsets, nseg, (cudaStream_t)st, 1);
}
int gms_segmented_sort_kv_f32_i32(const float* ki, const int32_t* vi, float* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint32_t, gms::FloatOrder32>, uint32_t, int32_t>(
      (const uint32_t*)ki, vi, (uint32_t*)ko, vo, n, offsets, nseg, (cudaStream_t)st, 2);
}
int gms_segmented_sort_kv_i64_i32(const int64_t* ki, const int32_t* vi, int64_t* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint64_t, gms::SignFlip64>, uint64_t, int32_t>(
      (const uint64_t*)ki, vi, (uint64_t*)ko, vo, n, offsets, nseg, (cudaStream_t)st, 3);
}
int gms_segmented_sort_kv_u64_i32(const uint64_t* ki, const int32_t* vi, uint64_t* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t, int32_t>(
      ki, vi, ko, vo, n, offsets, nseg, (cudaStream_t)st, 4);
}
int gms_segmented_sort_kv_f64_i32(const double* ki, const int32_t* vi, double* ko, int32_t* vo, int64_t n,
                                  const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<KvEngine<uint64_t, gms::FloatOrder64>, uint64_t, int32_t>(
      (const uint64_t*)ki, vi, (uint64_t*)ko, vo, n, offsets, nseg, (cudaStream_t)st, 5);
}

}  // extern "C"
