// Shared plumbing of the C ABI (include/gms.h): status/error recording, the
// per-(device, stream) scratch cache, and the engine instantiations used by
// the prebuilt dtypes.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <type_traits>

#include "../../include/gms.h"
#include "gms_engines.cuh"
#include "gms_sort.cuh"

namespace gms_capi {

using gms_engines::IndexGeo;
using gms_engines::KeysEngine;
using gms_engines::KeysGeo;
using gms_engines::KeysIndexGeo;
using gms_engines::KvEngine;
using gms_engines::kItems;
using gms_engines::kNT;

// Smallest forecast-tile capacity of any prebuilt engine: a tuning must leave
// room for a tile in every one (capacity / sample_b > k).
constexpr int kMinTileCap = IndexGeo::CAPW;

// error recording (defined in gms_capi_misc.cu)
int set_error(int status, const char* msg);
int cuda_error(cudaError_t e, const char* where);
void clear_error();

// Instrumentation must not record events while a stream is being captured.
int timing_suspend();
void timing_resume(int was_on);

// Scratch cache.  `tag` separates independent buffers of one call.
void* cache_get(int tag, size_t bytes, cudaStream_t st, int* status);

// Tuning used by a call: the tuning set with gms_set_tune if the caller set
// one; else the autotuned entry for (dtype, payload, size class) if there is
// one; else the defaults gms::Tune{}.
gms::Tune current_tune();
gms::Tune tune_for(int dtype, int kv, int64_t n);
// The tuning of a batch of arrays (n keys in all, the longest `longest`
// keys): an explicit or autotuned tuning of n's size class, else the
// built-in one for the longest array (its rounds are the batch's rounds).
gms::Tune tune_for_batch(int dtype, int kv, int64_t n, int64_t longest);
inline gms::Tune default_tune() { return current_tune(); }

// Frees the host-sort pipelines (streams, events, staging buffers).
void release_host_pipes();
// Forgets the per-device addresses of the allocation-free sort's static array.
void release_noalloc_symbols();

// Sorts with caller-provided scratch (gms_sort_ws); defined per key width.
int sort32_ws(int dtype, void* in, void* out, int64_t n, void* ws, size_t ws_bytes, cudaStream_t st);
int sort64_ws(int dtype, void* in, void* out, int64_t n, void* ws, size_t ws_bytes, cudaStream_t st);
int sort_kv_ws(int dtype, void* ki, int32_t* vi, void* ko, int32_t* vo, int64_t n, void* ws, size_t ws_bytes,
               cudaStream_t st);

// Runs a full sort of one dtype, with the scratch cache or, when `user_ws` is
// given, with the caller's scratch (its status word cleared first).
template <class Eng, class K, class V>
int run_sort(K* in, V* vin, K* out, V* vout, int64_t n, cudaStream_t st, int dtype, void* user_ws = nullptr,
             size_t user_bytes = 0, const gms::BaseGate* gate = nullptr, const gms::RoundSplit* split = nullptr) {
  clear_error();
  if (n < 0) return set_error(GMS_ERR_INVALID, "n < 0");
  if (n == 0) return GMS_OK;
  if (!in || !out) return set_error(GMS_ERR_INVALID, "null key pointer");
  if (gms::HasVal<V>::value && (!vin || !vout)) return set_error(GMS_ERR_INVALID, "null value pointer");
  if (n > ((int64_t)1 << 32) * 32) return set_error(GMS_ERR_TOO_LARGE, "n beyond 2^37");
  const gms::Tune t = tune_for(dtype, gms::HasVal<V>::value ? 1 : 0, n);
  const gms::WsLayout l = Eng::plan(n, t);
  if (!l.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this n (sample recursion too deep)");
  const size_t bytes = gms::ws_bytes_for<K>(l, t.k);
  int status = GMS_OK;
  void* ws = nullptr;
  if (user_ws) {
    if (user_bytes < bytes) {
      char msg[128];
      snprintf(msg, sizeof(msg), "workspace too small: %zu bytes given, %zu needed", user_bytes, bytes);
      return set_error(GMS_ERR_INVALID, msg);
    }
    if (reinterpret_cast<uintptr_t>(user_ws) % 256) return set_error(GMS_ERR_INVALID, "workspace not 256-byte aligned");
    cudaError_t e = cudaMemsetAsync(user_ws, 0, 256, st);
    if (e != cudaSuccess) return cuda_error(e, "workspace status word");
    ws = user_ws;
  } else {
    ws = cache_get(0, bytes, st, &status);
    if (status != GMS_OK) return status;
  }
  const gms::WsPtrs<K> w = gms::ws_carve<K>(l, t.k, ws);
  gms::BaseGate g2;
  if (gate && gate->side) {
    // a second scratch of the same layout for the odd chunks' level buffers
    g2 = *gate;
    g2.alt_ws = cache_get(41, bytes, st, &status);
    if (status != GMS_OK) return status;
    gate = &g2;
  }
  cudaError_t e = Eng::sort(w, in, vin, out, vout, n, t, st, gate, split);
  if (e != cudaSuccess) return cuda_error(e, "sort");
  return GMS_OK;
}

template <class Eng, class K>
size_t sort_ws_bytes(int64_t n, int dtype, int kv) {
  const gms::Tune t = tune_for(dtype, kv, n);
  return gms::ws_bytes_for<K>(Eng::plan(n, t), t.k);
}

}  // namespace gms_capi
