// C ABI: 32-bit keys (int32, uint32, float32), keys only.
#include "gms_capi.cuh"

using namespace gms_capi;
using gms::NoVal;

namespace {

using EngI32 = KeysEngine<uint32_t, gms::SignFlip32>;
using EngU32 = KeysEngine<uint32_t, gms::IdentityCodec<uint32_t>>;
using EngF32 = KeysEngine<uint32_t, gms::FloatOrder32>;

template <class Eng>
int sort32(void* in, void* out, int64_t n, void* st, int dtype) {
  return run_sort<Eng, uint32_t, NoVal>((uint32_t*)in, nullptr, (uint32_t*)out, nullptr, n, (cudaStream_t)st, dtype);
}

}  // namespace

int gms_capi::sort32_ws(int dtype, void* in, void* out, int64_t n, void* ws, size_t bytes, cudaStream_t st) {
  uint32_t* i = (uint32_t*)in;
  uint32_t* o = (uint32_t*)out;
  switch (dtype) {
    case 0: return run_sort<EngI32, uint32_t, NoVal>(i, nullptr, o, nullptr, n, st, 0, ws, bytes);
    case 1: return run_sort<EngU32, uint32_t, NoVal>(i, nullptr, o, nullptr, n, st, 1, ws, bytes);
    default: return run_sort<EngF32, uint32_t, NoVal>(i, nullptr, o, nullptr, n, st, 2, ws, bytes);
  }
}

extern "C" {

int gms_sort_i32(int32_t* in, int32_t* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort32<EngI32>(in, out, n, st, 0);
}
int gms_sort_u32(uint32_t* in, uint32_t* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort32<EngU32>(in, out, n, st, 1);
}
int gms_sort_f32(float* in, float* out, int64_t n, int tb, void* st) {
  (void)tb;
  return sort32<EngF32>(in, out, n, st, 2);
}

int gms_tile_sort_i32(int32_t* data, int64_t n, int64_t tile, void* st) {
  clear_error();
  if (n < 0 || tile < 1 || tile > EngI32::CAP) return set_error(GMS_ERR_INVALID, "bad n or tile");
  if (n == 0) return GMS_OK;
  if (!data) return set_error(GMS_ERR_INVALID, "null pointer");
  cudaError_t e = EngI32::tile_sort((uint32_t*)data, n, tile, (cudaStream_t)st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "tile_sort");
}

int gms_merge_level_i32(const int32_t* in, int32_t* out, int64_t n, int64_t run_len, int k, void* st) {
  clear_error();
  if (n < 0 || run_len < 1 || k < 2 || k > 32) return set_error(GMS_ERR_INVALID, "bad n, run_len or k");
  if (n == 0) return GMS_OK;
  if (!in || !out) return set_error(GMS_ERR_INVALID, "null pointer");
  gms::Tune t = default_tune();
  t.k = k;
  const gms::WsLayout l = EngI32::plan_merge_level(n, run_len, t);
  if (!l.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this n (sample recursion too deep)");
  int status = GMS_OK;
  void* ws = cache_get(0, gms::ws_bytes_for<uint32_t>(l, k), (cudaStream_t)st, &status);
  if (status != GMS_OK) return status;
  const gms::WsPtrs<uint32_t> w = gms::ws_carve<uint32_t>(l, k, ws);
  cudaError_t e = EngI32::merge_level(w, (const uint32_t*)in, (uint32_t*)out, n, run_len, t, (cudaStream_t)st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "merge_level");
}

int gms_find_partitions_i32(const int32_t* task, int64_t size, int k, int64_t task_size, const int64_t* ranks,
                            int64_t nranks, int64_t* out, void* stv) {
  clear_error();
  if (size < 1 || k < 1 || k > 32 || task_size < 0 || task_size > size * k || nranks < 0)
    return set_error(GMS_ERR_INVALID, "bad size, k, task_size or nranks");
  if (nranks == 0) return GMS_OK;
  if (!task || !ranks || !out) return set_error(GMS_ERR_INVALID, "null pointer");
  if (task_size > 0xffffffffll) return set_error(GMS_ERR_TOO_LARGE, "task_size beyond 2^32");
  cudaStream_t st = (cudaStream_t)stv;
  gms::Tune t = default_tune();
  t.k = k < 2 ? 2 : k;
  int status = GMS_OK;
  const size_t mk_bytes = gms::align_up(sizeof(uint32_t) * (size_t)(task_size + 1), 256);
  char* tmp = (char*)cache_get(1, 2 * mk_bytes, st, &status);
  if (status != GMS_OK) return status;
  uint32_t* mk = (uint32_t*)tmp;
  uint32_t* mi = (uint32_t*)(tmp + mk_bytes);
  cudaError_t e = cudaSuccess;
  if (task_size > 0) {
    const gms::WsLayout l = EngI32::plan_merge_level(task_size, size, t);
    if (!l.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this task (sample recursion too deep)");
    void* ws = cache_get(0, gms::ws_bytes_for<uint32_t>(l, t.k), st, &status);
    if (status != GMS_OK) return status;
    const gms::WsPtrs<uint32_t> w = gms::ws_carve<uint32_t>(l, t.k, ws);
    // merge the task keeping each key's origin; keys stay encoded
    e = EngI32::round<uint32_t>(w, 0, (const uint32_t*)task, nullptr, mk, mi, task_size, size, t, nullptr, nullptr, 1,
                                0, 1, st);
    if (e != cudaSuccess) return cuda_error(e, "find_partitions merge");
  }
  const int64_t threads = nranks * 32;
  gms::hook_before(gms::KC_CORANK, st);
  gms::corank_kernel<uint32_t, gms::KeyLess, gms::SignFlip32>
      <<<(unsigned)gms::ceil_div(threads, 256), 256, 0, st>>>((const uint32_t*)task, mk, mi, size, k, task_size, ranks,
                                                               nranks, out);
  e = cudaGetLastError();
  gms::hook_after(gms::KC_CORANK, st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "corank_kernel");
}

int gms_sort_host_i32(const int32_t* host_in, int32_t* host_out, int64_t n, void* stv) {
  clear_error();
  if (n < 0) return set_error(GMS_ERR_INVALID, "n < 0");
  if (n == 0) return GMS_OK;
  if (!host_in || !host_out) return set_error(GMS_ERR_INVALID, "null pointer");
  cudaStream_t st = (cudaStream_t)stv;
  int status = GMS_OK;
  const size_t bytes = sizeof(int32_t) * (size_t)n;
  void* din = cache_get(10, bytes, st, &status);
  if (status != GMS_OK) return status;
  void* dout = cache_get(11, bytes, st, &status);
  if (status != GMS_OK) return status;
  cudaError_t e = cudaMemcpyAsync(din, host_in, bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync H2D");
  status = sort32<EngI32>(din, dout, n, st, 0);
  if (status != GMS_OK) return status;
  e = cudaMemcpyAsync(host_out, dout, bytes, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync D2H");
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "cudaStreamSynchronize");
}

}  // extern "C"
