// C ABI: an int32 sort that allocates nothing.
//
// Some callers cannot allocate device memory once they are running: a
// latency-critical serving loop, where cudaMalloc/cudaFree can synchronize the
// device and stall every other stream; or a host framework that hands each
// plugin a fixed memory budget at start-up and forbids allocation inside its
// callbacks.  gms_sort_i32 draws scratch from a cache that grows with
// cudaMalloc, so it does not suit them.  gms_sort_i32_noalloc runs the same
// sort with its scratch in a file-scope device array of fixed size instead.
//
//   * The array (kNoallocScratchBytes, 4 MiB) is static device memory: every
//     GPU that loads this library holds it until the process exits.
//   * It covers n <= GMS_NOALLOC_MAX_N (2^22 keys) with the default tuning
//     (fan-in 32, sample block 32), which this entry point always uses,
//     whatever gms_set_tune has set.  Larger n is rejected.
//   * Host code cannot pass the array's name to a kernel (on the host it is
//     only a stand-in symbol), so the device address is looked up with
//     cudaGetSymbolAddress, once per device, on the first call made while
//     that device is current.  Make that first call before any stream capture.
//   * Every call uses the same array, and the array keeps the last call's
//     contents.  Only the status word at its start must begin at zero; it is
//     cleared on the caller's stream at the start of each call.  Calls whose
//     work overlaps on the GPU (different streams, or different host threads
//     without ordering) race on the array: order them.
#include <mutex>

#include "gms_capi.cuh"

using namespace gms_capi;

namespace {

constexpr size_t kNoallocScratchBytes = size_t(4) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

using EngNoalloc = KeysEngine<uint32_t, gms::SignFlip32>;

std::mutex g_sym_mu;
void* g_sym_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_ptr(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return set_error(GMS_ERR_INVALID, "device ordinal beyond 63");
  std::lock_guard<std::mutex> g(g_sym_mu);
  if (!g_sym_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_sym_ptr[dev] = p;
  }
  *out = g_sym_ptr[dev];
  return GMS_OK;
}

}  // namespace

namespace gms_capi {
void release_noalloc_symbols() {
  std::lock_guard<std::mutex> g(g_sym_mu);
  for (void*& p : g_sym_ptr) p = nullptr;
}
}  // namespace gms_capi

extern "C" {

int gms_sort_i32_noalloc(int32_t* input, int32_t* output, int64_t n, void* stream) {
  clear_error();
  if (n < 0) return set_error(GMS_ERR_INVALID, "n < 0");
  if (n > GMS_NOALLOC_MAX_N)
    return set_error(GMS_ERR_TOO_LARGE, "gms_sort_i32_noalloc: n exceeds GMS_NOALLOC_MAX_N (2^22 keys)");
  if (n == 0) return GMS_OK;
  if (!input || !output) return set_error(GMS_ERR_INVALID, "null pointer");
  const gms::Tune t;  // default tuning: the size bound below is computed for it
  const gms::WsLayout l = EngNoalloc::plan(n, t);
  const size_t need = gms::ws_bytes_for<uint32_t>(l, t.k);
  if (!l.ok || need > kNoallocScratchBytes)
    return set_error(GMS_ERR_TOO_LARGE, "gms_sort_i32_noalloc: scratch need exceeds the static array");
  void* ws = nullptr;
  int status = scratch_ptr(&ws);
  if (status != GMS_OK) return status;
  cudaStream_t st = (cudaStream_t)stream;
  // the status word is the only scratch that must start at zero
  cudaError_t e = cudaMemsetAsync(ws, 0, 256, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync(status word)");
  const gms::WsPtrs<uint32_t> w = gms::ws_carve<uint32_t>(l, t.k, ws);
  e = EngNoalloc::sort(w, (uint32_t*)input, nullptr, (uint32_t*)output, nullptr, n, t, st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "gms_sort_i32_noalloc");
}

int gms_noalloc_status(void* stream, int* status_out) {
  clear_error();
  if (!status_out) return set_error(GMS_ERR_INVALID, "null status_out");
  *status_out = 0;
  void* ws = nullptr;
  int status = scratch_ptr(&ws);
  if (status != GMS_OK) return status;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  // a synchronous copy into a host variable: no staging buffer of ours
  int v = 0;
  e = cudaMemcpy(&v, ws, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "noalloc status word");
  *status_out = v;
  return GMS_OK;
}

}  // extern "C"
