// C ABI: version, status strings, error recording, scratch cache, queries.
#include <algorithm>
#include <mutex>
#include <vector>

#include "gms_capi.cuh"

namespace gms_capi {

static thread_local std::string g_last_error;

int set_error(int status, const char* msg) {
  g_last_error = msg ? msg : "";
  return status;
}
int cuda_error(cudaError_t e, const char* where) {
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
  g_last_error = buf;
  return e == cudaErrorMemoryAllocation ? GMS_ERR_NOMEM : GMS_ERR_CUDA;
}
void clear_error() { g_last_error.clear(); }

namespace {
struct Slot {
  int dev;
  cudaStream_t stream;
  int tag;
  void* ptr;
  size_t bytes;
};
std::mutex g_mu;
std::vector<Slot> g_slots;
}  // namespace

void* cache_get(int tag, size_t bytes, cudaStream_t st, int* status) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *status = cuda_error(e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_mu);
  for (Slot& s : g_slots) {
    if (s.dev == dev && s.stream == st && s.tag == tag) {
      if (s.bytes >= bytes) return s.ptr;
      // grow: the previous call on this stream may still use the buffer
      e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        *status = cuda_error(e, "cudaStreamSynchronize");
        return nullptr;
      }
      cudaFree(s.ptr);
      s.ptr = nullptr;
      s.bytes = 0;
      e = cudaMalloc(&s.ptr, bytes);
      if (e != cudaSuccess) {
        s.ptr = nullptr;
        *status = cuda_error(e, "cudaMalloc(scratch)");
        return nullptr;
      }
      s.bytes = bytes;
      cudaMemset(s.ptr, 0, bytes < 256 ? bytes : 256);  // status word starts clear
      return s.ptr;
    }
  }
  void* p = nullptr;
  e = cudaMalloc(&p, bytes > 0 ? bytes : 256);
  if (e != cudaSuccess) {
    *status = cuda_error(e, "cudaMalloc(scratch)");
    return nullptr;
  }
  cudaMemset(p, 0, 256);  // status word starts clear
  g_slots.push_back(Slot{dev, st, tag, p, bytes > 0 ? bytes : 256});
  return p;
}

// ---- launch counting and live kernel timing ----
namespace {
struct TimedLaunch {
  int kc;
  cudaEvent_t a, b;
};
std::mutex g_prof_mu;
long long g_launches[gms::KC_COUNT] = {0};
int g_timing = 0;
std::vector<TimedLaunch> g_pending;
std::vector<cudaEvent_t> g_event_pool;
double g_ms[gms::KC_COUNT] = {0};
long long g_timed[gms::KC_COUNT] = {0};
// the open event of each class, per host thread (launches from several
// threads with timing on pair their own events)
thread_local cudaEvent_t t_open[gms::KC_COUNT];

cudaEvent_t pool_event() {
  if (!g_event_pool.empty()) {
    cudaEvent_t e = g_event_pool.back();
    g_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void before_launch(int kc, cudaStream_t st) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  if (!g_timing) return;
  t_open[kc] = pool_event();
  cudaEventRecord(t_open[kc], st);
}
void after_launch(int kc, cudaStream_t st) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  if (kc < gms::KC_H2D) g_launches[kc]++;  // the copy classes are not kernels
  cudaEvent_t a = t_open[kc];
  t_open[kc] = nullptr;
  if (!a) return;  // timing was off when the launch began
  if (!g_timing) {  // and was switched off since
    g_event_pool.push_back(a);
    return;
  }
  cudaEvent_t b = pool_event();
  cudaEventRecord(b, st);
  g_pending.push_back(TimedLaunch{kc, a, b});
}
gms::Hooks g_hook_table{before_launch, after_launch};
}  // namespace

int timing_suspend() {
  std::lock_guard<std::mutex> g(g_prof_mu);
  const int was = g_timing;
  g_timing = 0;
  return was;
}
void timing_resume(int was_on) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_timing = was_on;
}

namespace {
struct InstallHooks {
  InstallHooks() { gms::g_hooks = &g_hook_table; }
} g_install_hooks;
}  // namespace

}  // namespace gms_capi

using namespace gms_capi;

extern "C" {

int gms_version(void) { return 100; }

const char* gms_status_string(int s) {
  switch (s) {
    case GMS_OK: return "GMS_OK";
    case GMS_ERR_INVALID: return "GMS_ERR_INVALID";
    case GMS_ERR_CUDA: return "GMS_ERR_CUDA";
    case GMS_ERR_NOMEM: return "GMS_ERR_NOMEM";
    case GMS_ERR_TOO_LARGE: return "GMS_ERR_TOO_LARGE";
    case GMS_ERR_INTERNAL: return "GMS_ERR_INTERNAL";
    default: return "GMS_ERR_UNKNOWN";
  }
}

const char* gms_last_error(void) { return g_last_error.c_str(); }

int gms_set_pdl(int on) {
  clear_error();
  if (on != 0 && on != 1) return set_error(GMS_ERR_INVALID, "gms_set_pdl takes 0 or 1");
  gms::pdl_enabled().store(on, std::memory_order_relaxed);
  return GMS_OK;
}

int gms_get_pdl(void) { return gms::pdl_enabled().load(std::memory_order_relaxed); }

void gms_release_workspaces(void) {
  release_host_pipes();
  release_noalloc_symbols();
  std::lock_guard<std::mutex> g(g_mu);
  for (Slot& s : g_slots) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(s.dev);
    cudaFree(s.ptr);
    cudaSetDevice(cur);
  }
  g_slots.clear();
}

long long gms_launch_count(void) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  long long t = 0;
  for (int i = 0; i < gms::KC_COUNT; ++i) t += g_launches[i];
  return t;
}

int gms_timing_enable(int on) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  g_timing = on ? 1 : 0;
  return GMS_OK;
}

int gms_timing_collect(double* ms, long long* launches, int nclasses) {
  clear_error();
  std::lock_guard<std::mutex> g(g_prof_mu);
  for (const TimedLaunch& t : g_pending) {
    float f = 0.f;
    cudaError_t e = cudaEventSynchronize(t.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, t.a, t.b);
    if (e != cudaSuccess) return cuda_error(e, "cudaEventElapsedTime");
    g_ms[t.kc] += f;
    g_timed[t.kc] += 1;
    g_event_pool.push_back(t.a);
    g_event_pool.push_back(t.b);
  }
  g_pending.clear();
  for (int i = 0; i < nclasses && i < gms::KC_COUNT; ++i) {
    if (ms) ms[i] = g_ms[i];
    if (launches) launches[i] = g_timed[i];
  }
  return GMS_OK;
}

int gms_timing_trace(int* classes, double* start_ms, double* end_ms, int max_entries) {
  clear_error();
  std::lock_guard<std::mutex> g(g_prof_mu);
  const int n = (int)g_pending.size();
  if (n == 0) return 0;
  // times relative to the first recorded start, shifted so the earliest is 0
  std::vector<float> a(n), b(n);
  for (int i = 0; i < n; ++i) {
    cudaError_t e = cudaEventSynchronize(g_pending[i].b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&a[i], g_pending[0].a, g_pending[i].a);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b[i], g_pending[0].a, g_pending[i].b);
    if (e != cudaSuccess) return cuda_error(e, "cudaEventElapsedTime");
  }
  float lo = 0.f;
  for (int i = 0; i < n; ++i) lo = std::min(lo, a[i]);
  for (int i = 0; i < n && i < max_entries; ++i) {
    if (classes) classes[i] = g_pending[i].kc;
    if (start_ms) start_ms[i] = a[i] - lo;
    if (end_ms) end_ms[i] = b[i] - lo;
  }
  return n;
}

int gms_timing_reset(void) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  for (int i = 0; i < gms::KC_COUNT; ++i) {
    g_ms[i] = 0;
    g_timed[i] = 0;
  }
  return GMS_OK;
}

int64_t gms_max_tile(void) { return (int64_t)kNT * kItems; }

int64_t gms_base_tile(int dtype, int kv) {
  if (kv) return KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>::BASE_TILE;
  if (dtype >= 3) return KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>::BASE_TILE;
  return KeysEngine<uint32_t, gms::IdentityCodec<uint32_t>>::BASE_TILE;
}

int gms_rounds(int dtype, int kv, int64_t n) {
  const gms::Tune t = tune_for(dtype, kv, n);
  if (kv) return KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>::passes_for(n, t);
  if (dtype >= 3) return KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>::passes_for(n, t);
  return KeysEngine<uint32_t, gms::IdentityCodec<uint32_t>>::passes_for(n, t);
}

size_t gms_workspace_bytes(int dtype, int kv, int64_t n) {
  if (n <= 0) return 0;
  const bool wide = (dtype >= 3);
  if (wide) {
    return kv ? sort_ws_bytes<KvEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t>(n, dtype, kv)
              : sort_ws_bytes<KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>, uint64_t>(n, dtype, kv);
  }
  return kv ? sort_ws_bytes<KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>, uint32_t>(n, dtype, kv)
            : sort_ws_bytes<KeysEngine<uint32_t, gms::IdentityCodec<uint32_t>>, uint32_t>(n, dtype, kv);
}

int gms_device_status(void* stream, int* status_out) {
  clear_error();
  if (!status_out) return set_error(GMS_ERR_INVALID, "null status_out");
  *status_out = 0;
  cudaStream_t st = (cudaStream_t)stream;
  int status = GMS_OK;
  void* ws = cache_get(0, 256, st, &status);
  if (status != GMS_OK) return status;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  int v = 0;
  e = cudaMemcpy(&v, ws, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(ws, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_error(e, "status word");
  *status_out = v;
  return GMS_OK;
}

int gms_sort_ws(int dtype, int kv, void* keys_in, int32_t* vals_in, void* keys_out, int32_t* vals_out, int64_t n,
                void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  if (dtype < 0 || dtype > 5 || (kv != 0 && kv != 1)) return set_error(GMS_ERR_INVALID, "dtype in 0..5, kv 0 or 1");
  if (!workspace) return set_error(GMS_ERR_INVALID, "null workspace");
  cudaStream_t st = (cudaStream_t)stream;
  if (kv) return sort_kv_ws(dtype, keys_in, vals_in, keys_out, vals_out, n, workspace, workspace_bytes, st);
  if (dtype < 3) return sort32_ws(dtype, keys_in, keys_out, n, workspace, workspace_bytes, st);
  return sort64_ws(dtype, keys_in, keys_out, n, workspace, workspace_bytes, st);
}

int gms_workspace_status(void* workspace, void* stream, int* status_out) {
  clear_error();
  if (!workspace || !status_out) return set_error(GMS_ERR_INVALID, "null pointer");
  *status_out = 0;
  cudaStream_t st = (cudaStream_t)stream;
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, workspace, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemsetAsync(workspace, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_error(e, "workspace status word");
  *status_out = v;
  return GMS_OK;
}

int gms_reserve(int dtype, int kv, int64_t n, void* stream) {
  clear_error();
  if (dtype < 0 || dtype > GMS_RESERVE_SEGMENTED_I32 || n < 0) return set_error(GMS_ERR_INVALID, "bad dtype or n");
  int status = GMS_OK;
  if (dtype == GMS_RESERVE_SEGMENTED_I32) {
    // a plain sort's scratch and the batched sort's scratch array of n keys
    cache_get(0, gms_workspace_bytes(0, 0, n), (cudaStream_t)stream, &status);
    if (status == GMS_OK) cache_get(30, sizeof(uint32_t) * (size_t)(n > 0 ? n : 1), (cudaStream_t)stream, &status);
    return status;
  }
  cache_get(0, gms_workspace_bytes(dtype, kv, n), (cudaStream_t)stream, &status);
  return status;
}

}  // extern "C"
