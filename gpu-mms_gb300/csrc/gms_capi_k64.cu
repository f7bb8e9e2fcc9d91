// C ABI: 64-bit keys (int64, uint64, float64), keys only.
#include "gms_capi.cuh"
#include "gms_capi_seg.cuh"

using namespace gms_capi;
using gms::NoVal;

namespace {

using EngI64 = KeysEngine<uint64_t, gms::SignFlip64>;
using EngU64 = KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>;
using EngF64 = KeysEngine<uint64_t, gms::FloatOrder64>;

template <class Eng>
int sort64(void* in, void* out, int64_t n, void* st, int dtype) {
  return run_sort<Eng, uint64_t, NoVal>((uint64_t*)in, nullptr, (uint64_t*)out, nullptr, n, (cudaStream_t)st, dtype);
}

}  // namespace

int gms_capi::sort64_ws(int dtype, void* in, void* out, int64_t n, void* ws, size_t bytes, cudaStream_t st) {
  uint64_t* i = (uint64_t*)in;
  uint64_t* o = (uint64_t*)out;
  switch (dtype) {
    case 3: return run_sort<EngI64, uint64_t, NoVal>(i, nullptr, o, nullptr, n, st, 3, ws, bytes);
    case 4: return run_sort<EngU64, uint64_t, NoVal>(i, nullptr, o, nullptr, n, st, 4, ws, bytes);
    default: return run_sort<EngF64, uint64_t, NoVal>(i, nullptr, o, nullptr, n, st, 5, ws, bytes);
  }
}

extern "C" {

int gms_sort_i64(int64_t* in, int64_t* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort64<EngI64>(in, out, n, st, 3);
}
int gms_sort_u64(uint64_t* in, uint64_t* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort64<EngU64>(in, out, n, st, 4);
}
int gms_sort_f64(double* in, double* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort64<EngF64>(in, out, n, st, 5);
}

int gms_tile_sort_u64(uint64_t* data, int64_t n, int64_t tile, void* st) {
  clear_error();
  if (n < 0 || tile < 1 || tile > EngU64::CAP) return set_error(GMS_ERR_INVALID, "bad n or tile");
  if (n == 0) return GMS_OK;
  if (!data) return set_error(GMS_ERR_INVALID, "null pointer");
  cudaError_t e = EngU64::tile_sort(data, n, tile, (cudaStream_t)st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "tile_sort");
}

int gms_merge_level_u64(const uint64_t* in, uint64_t* out, int64_t n, int64_t run_len, int k, void* st) {
  clear_error();
  if (n < 0 || run_len < 1 || k < 2 || k > 32) return set_error(GMS_ERR_INVALID, "bad n, run_len or k");
  if (n == 0) return GMS_OK;
  if (!in || !out) return set_error(GMS_ERR_INVALID, "null pointer");
  gms::Tune t = default_tune();
  t.k = k;
  const gms::WsLayout l = EngU64::plan_merge_level(n, run_len, t);
  if (!l.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this n (sample recursion too deep)");
  int status = GMS_OK;
  void* ws = cache_get(0, gms::ws_bytes_for<uint64_t>(l, k), (cudaStream_t)st, &status);
  if (status != GMS_OK) return status;
  const gms::WsPtrs<uint64_t> w = gms::ws_carve<uint64_t>(l, k, ws);
  cudaError_t e = EngU64::merge_level(w, in, out, n, run_len, t, (cudaStream_t)st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "merge_level");
}

int gms_segmented_sort_i64(const int64_t* in, int64_t* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<EngI64, uint64_t, NoVal>((const uint64_t*)in, nullptr, (uint64_t*)out, nullptr, n, offsets, nseg,
                                                (cudaStream_t)st, 3);
}
int gms_segmented_sort_u64(const uint64_t* in, uint64_t* out, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* st) {
  return run_segmented<EngU64, uint64_t, NoVal>(in, nullptr, out, nullptr, n, offsets, nseg, (cudaStream_t)st, 4);
}
int gms_segmented_sort_f64(const double* in, double* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<EngF64, uint64_t, NoVal>((const uint64_t*)in, nullptr, (uint64_t*)out, nullptr, n, offsets, nseg,
                                                (cudaStream_t)st, 5);
}

}  // extern "C"
