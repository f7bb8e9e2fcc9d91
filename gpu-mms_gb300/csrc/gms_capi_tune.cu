// C ABI: tuning.  The process-wide tuning set by the caller (gms_set_tune), the
// autotuner (gms_autotune) that times candidate tunings for one (dtype,
// payload, size class) on the device and keeps the fastest in a table that
// later sorts of that class consult, and the table's JSON cache keyed by GPU
// name.
//
// Replaces the reference's compile-time constants K, PIPELINE and BLOCKS
// (src/params.h:18-20) and its sweep scripts (scripts/findK.sh,
// scripts/blocksThreads.sh), which rebuild and rerun testMM per candidate.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <vector>

#include "gms_capi.cuh"

namespace gms_capi {
namespace {

std::mutex g_tune_mu;
gms::Tune g_tune;
bool g_tune_explicit = false;  // gms_set_tune was called (wins over the table)

struct TuneEntry {
  int dtype, kv, cls;  // cls = floor(log2 n)
  gms::Tune t;
  double ms;           // median time of one sort of the tuned size
};
std::vector<TuneEntry> g_table;

// Set by the autotuner on its own thread while it times a candidate.
thread_local const gms::Tune* t_override = nullptr;
struct OverrideScope {
  explicit OverrideScope(const gms::Tune* t) { t_override = t; }
  ~OverrideScope() { t_override = nullptr; }
};

std::once_flag g_autoload_once;

int size_class(int64_t n) {
  int c = 0;
  while (n > 1) {
    n >>= 1;
    ++c;
  }
  return c;
}

bool valid_tune(int k, int sample_b) {
  return k >= 2 && k <= 32 && sample_b >= 8 && (int64_t)kMinTileCap / sample_b - k >= 1;
}

void table_put(int dtype, int kv, int cls, const gms::Tune& t, double ms) {
  for (TuneEntry& e : g_table) {
    if (e.dtype == dtype && e.kv == kv && e.cls == cls) {
      e.t = t;
      e.ms = ms;
      return;
    }
  }
  g_table.push_back(TuneEntry{dtype, kv, cls, t, ms});
}

int device_name(std::string* name) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  cudaDeviceProp p;
  e = cudaGetDeviceProperties(&p, dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceProperties");
  *name = p.name;
  return GMS_OK;
}

std::string json_escape(const std::string& s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    if ((unsigned char)c >= 0x20) o += c;
  }
  return o;
}

std::string table_json_locked() {
  std::string out = "[";
  char buf[256];
  for (size_t i = 0; i < g_table.size(); ++i) {
    const TuneEntry& e = g_table[i];
    snprintf(buf, sizeof(buf),
             "%s{\"dtype\": %d, \"kv\": %d, \"log2n\": %d, \"k\": %d, \"sample_b\": %d, \"bulk_copy\": %d, "
             "\"split\": %d, \"base\": %d, \"ms\": %.4f}",
             i ? ", " : "", e.dtype, e.kv, e.cls, e.t.k, e.t.sample_b, e.t.bulk_copy, e.t.split, e.t.base, e.ms);
    out += buf;
  }
  return out + "]";
}

// Value of integer field `key` inside one JSON object [p, q); false if absent.
bool field_num(const char* p, const char* q, const char* key, double* v) {
  const std::string pat = std::string("\"") + key + "\"";
  const char* f = std::search(p, q, pat.begin(), pat.end());
  if (f == q) return false;
  f += pat.size();
  while (f < q && (*f == ' ' || *f == ':')) ++f;
  char* end = nullptr;
  *v = strtod(f, &end);
  return end != f && end <= q;
}

// Parses a cache file.  The whole file is rejected (and the table left as it
// was) when the GPU name differs or any entry is malformed.
int load_cache(const char* path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return set_error(GMS_ERR_INVALID, "tune cache: cannot open file");
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  std::string dev;
  int status = device_name(&dev);
  if (status != GMS_OK) return status;
  const std::string want = "\"device\": \"" + json_escape(dev) + "\"";
  if (s.find(want) == std::string::npos) return set_error(GMS_ERR_INVALID, "tune cache: recorded for another GPU");
  const size_t lb = s.find('[');
  if (lb == std::string::npos) return set_error(GMS_ERR_INVALID, "tune cache: no entries list");
  std::vector<TuneEntry> got;
  size_t pos = lb;
  while (true) {
    const size_t a = s.find('{', pos);
    if (a == std::string::npos) break;
    const size_t b = s.find('}', a);
    if (b == std::string::npos) return set_error(GMS_ERR_INVALID, "tune cache: unterminated entry");
    const char* p = s.data() + a;
    const char* q = s.data() + b;
    double dt, kv, cls, k, sb, bulk, ms = 0;
    if (!field_num(p, q, "dtype", &dt) || !field_num(p, q, "kv", &kv) || !field_num(p, q, "log2n", &cls) ||
        !field_num(p, q, "k", &k) || !field_num(p, q, "sample_b", &sb) || !field_num(p, q, "bulk_copy", &bulk))
      return set_error(GMS_ERR_INVALID, "tune cache: entry lacks a field");
    field_num(p, q, "ms", &ms);
    double split = 0, base = 0;  // optional (files written before these choices existed lack them)
    field_num(p, q, "split", &split);
    field_num(p, q, "base", &base);
    if (dt < 0 || dt > 5 || (kv != 0 && kv != 1) || cls < 0 || cls > 40 || !valid_tune((int)k, (int)sb) ||
        bulk < 0 || bulk > 3 || (split != 0 && split != 1) || (base != 0 && base != 1))
      return set_error(GMS_ERR_INVALID, "tune cache: entry out of range");
    gms::Tune t;
    t.k = (int)k;
    t.sample_b = (int)sb;
    t.bulk_copy = (int)bulk;
    t.split = (int)split;
    t.base = (int)base;
    got.push_back(TuneEntry{(int)dt, (int)kv, (int)cls, t, ms});
    pos = b + 1;
  }
  std::lock_guard<std::mutex> g(g_tune_mu);
  for (const TuneEntry& e : got) table_put(e.dtype, e.kv, e.cls, e.t, e.ms);
  return GMS_OK;
}

// GMS_TUNE_CACHE names a cache loaded before the first sort (best effort: a
// missing file or another GPU's cache leaves the defaults).
void autoload() {
  std::call_once(g_autoload_once, [] {
    const char* p = getenv("GMS_TUNE_CACHE");
    if (p && *p) {
      std::ifstream probe(p);
      if (probe) load_cache(p);
    }
  });
}

// Synthetic keys of the tuned class: uniform bits for the integer dtypes,
// finite values in [-1, 1) for the float ones (a splitmix64 hash of the index).
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__global__ void fill_kernel(void* keys, int32_t* vals, int64_t n, int dtype, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h = mix64(seed ^ (uint64_t)i);
    switch (dtype) {
      case 0:
      case 1: ((uint32_t*)keys)[i] = (uint32_t)h; break;
      case 2: ((float*)keys)[i] = (float)((int64_t)(h >> 40) - (1ll << 23)) * (1.0f / (1 << 23)); break;
      case 3:
      case 4: ((uint64_t*)keys)[i] = h; break;
      default: ((double*)keys)[i] = (double)((int64_t)(h >> 11) - (1ll << 52)) * (1.0 / (double)(1ll << 52)); break;
    }
    if (vals) vals[i] = (int32_t)i;
  }
}
__global__ void differ_kernel(const uint32_t* a, const uint32_t* b, int64_t words, int* flag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) {
    if (a[i] != b[i]) {
      *flag = 1;
      return;
    }
  }
}

int run_one(int dtype, int kv, void* ki, int32_t* vi, void* ko, int32_t* vo, int64_t n, cudaStream_t st) {
  switch (dtype * 2 + kv) {
    case 0: return gms_sort_i32((int32_t*)ki, (int32_t*)ko, n, 0, st);
    case 1: return gms_sort_kv_i32_i32((int32_t*)ki, vi, (int32_t*)ko, vo, n, 0, st);
    case 2: return gms_sort_u32((uint32_t*)ki, (uint32_t*)ko, n, 0, st);
    case 3: return gms_sort_kv_u32_i32((uint32_t*)ki, vi, (uint32_t*)ko, vo, n, 0, st);
    case 4: return gms_sort_f32((float*)ki, (float*)ko, n, 0, st);
    case 5: return gms_sort_kv_f32_i32((float*)ki, vi, (float*)ko, vo, n, 0, st);
    case 6: return gms_sort_i64((int64_t*)ki, (int64_t*)ko, n, 0, st);
    case 7: return gms_sort_kv_i64_i32((int64_t*)ki, vi, (int64_t*)ko, vo, n, 0, st);
    case 8: return gms_sort_u64((uint64_t*)ki, (uint64_t*)ko, n, 0, st);
    case 9: return gms_sort_kv_u64_i32((uint64_t*)ki, vi, (uint64_t*)ko, vo, n, 0, st);
    case 10: return gms_sort_f64((double*)ki, (double*)ko, n, 0, st);
    default: return gms_sort_kv_f64_i32((double*)ki, vi, (double*)ko, vo, n, 0, st);
  }
}

// Device buffers of one autotune call, freed on every exit path.
struct TuneBuffers {
  void* p[8] = {nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~TuneBuffers() {
    for (void* q : p)
      if (q) cudaFree(q);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};

}  // namespace

gms::Tune current_tune() {
  std::lock_guard<std::mutex> g(g_tune_mu);
  return g_tune;
}

// Built-in tuning of a class when neither gms_set_tune nor the autotuned
// table says otherwise (timed on GB300).
//   Staging (2^27 keys): sorts with a payload and sorts of 64-bit keys merge
//   faster with persistent CTAs that stage the next tile while storing the
//   current one (float32 + int32 -2%, uint64 + int32 -4%, uint64 keys alone
//   -2%: 7.90 against 8.08 ms); sorts of 32-bit keys alone do not (+1%).
//   Fan-in: gms_engines::balanced_fan_in.  A fan-in of 32 on 2048 base runs
//   (int32, 2^24 keys) would spend its third round merging 2 runs; 16 gives
//   three even rounds: 0.49 against 0.60 ms (int32 2^20: 0.109 against
//   0.124; uint64 2^24: 0.92 against 1.06, 2^18: fan-in 8, 0.081 against
//   0.118 ms; float32 + int32 2^24: fan-in 16, 0.88 against 1.01, 2^18:
//   fan-in 8, 0.077 against 0.106 ms), while 2^22, 2^26 and 2^28 keep 32
//   (their rounds are even).
gms::Tune builtin_tune(int dtype, int kv, int64_t n) {
  gms::Tune t;
  if (kv || dtype >= 3) t.bulk_copy = 3;  // dtypes 3-5: int64, uint64, float64
  if (!kv) {
    const int64_t base = dtype >= 3 ? (int64_t)KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>::BASE_TILE
                                    : (int64_t)KeysEngine<uint32_t, gms::IdentityCodec<uint32_t>>::BASE_TILE;
    t = gms_engines::balanced_fan_in(n, base, t);
  } else {
    t = gms_engines::balanced_fan_in(n, (int64_t)KvEngine<uint32_t, gms::IdentityCodec<uint32_t>>::BASE_TILE, t, 16);
  }
  return t;
}

gms::Tune tune_for(int dtype, int kv, int64_t n) { return tune_for_batch(dtype, kv, n, n); }

gms::Tune tune_for_batch(int dtype, int kv, int64_t n, int64_t longest) {
  if (t_override) return *t_override;
  autoload();
  std::lock_guard<std::mutex> g(g_tune_mu);
  if (g_tune_explicit) return g_tune;
  const int c = size_class(n);
  for (const TuneEntry& e : g_table)
    if (e.dtype == dtype && e.kv == kv && e.cls == c) return e.t;
  return builtin_tune(dtype, kv, longest);
}

}  // namespace gms_capi

using namespace gms_capi;

extern "C" {

int gms_set_tune(int k, int sample_b, int bulk_copy) {
  clear_error();
  if (k < 2 || k > 32) return set_error(GMS_ERR_INVALID, "k must be in [2, 32]");
  if (!valid_tune(k, sample_b))
    return set_error(GMS_ERR_INVALID, "sample_b must be >= 8 and leave room for a tile (4080/sample_b > k)");
  if (bulk_copy < 0 || bulk_copy > 3) return set_error(GMS_ERR_INVALID, "bulk_copy must be in [0, 3]");
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune.k = k;
  g_tune.sample_b = sample_b;
  g_tune.bulk_copy = bulk_copy;
  g_tune.split = 0;
  g_tune.base = 0;
  g_tune_explicit = true;
  return GMS_OK;
}

int gms_set_tune_ex(int k, int sample_b, int bulk_copy, int split, int base) {
  clear_error();
  if (split != 0 && split != 1) return set_error(GMS_ERR_INVALID, "split must be 0 or 1");
  if (base != 0 && base != 1) return set_error(GMS_ERR_INVALID, "base must be 0 or 1");
  const int rc = gms_set_tune(k, sample_b, bulk_copy);
  if (rc != GMS_OK) return rc;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune.split = split;
  g_tune.base = base;
  return GMS_OK;
}

int gms_get_tune_ex(int* k, int* sample_b, int* bulk_copy, int* split, int* base) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  if (k) *k = g_tune.k;
  if (sample_b) *sample_b = g_tune.sample_b;
  if (bulk_copy) *bulk_copy = g_tune.bulk_copy;
  if (split) *split = g_tune.split;
  if (base) *base = g_tune.base;
  return GMS_OK;
}

int gms_clear_tune(void) {
  clear_error();
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune = gms::Tune{};
  g_tune_explicit = false;
  return GMS_OK;
}

int gms_get_tune(int* k, int* sample_b, int* bulk_copy) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  if (k) *k = g_tune.k;
  if (sample_b) *sample_b = g_tune.sample_b;
  if (bulk_copy) *bulk_copy = g_tune.bulk_copy;
  return GMS_OK;
}

int gms_tune_for(int dtype, int kv, int64_t n, int* k, int* sample_b, int* bulk_copy) {
  clear_error();
  if (dtype < 0 || dtype > 5 || (kv != 0 && kv != 1)) return set_error(GMS_ERR_INVALID, "dtype in 0..5, kv 0 or 1");
  const gms::Tune t = tune_for(dtype, kv, n);
  if (k) *k = t.k;
  if (sample_b) *sample_b = t.sample_b;
  if (bulk_copy) *bulk_copy = t.bulk_copy;
  return GMS_OK;
}

int gms_autotune(int dtype, int kv, int64_t n, void* stream, int* out_k, int* out_sample_b, int* out_bulk_copy,
                 double* out_ms) {
  clear_error();
  if (dtype < 0 || dtype > 5 || (kv != 0 && kv != 1)) return set_error(GMS_ERR_INVALID, "dtype in 0..5, kv 0 or 1");
  if (n < 1) return set_error(GMS_ERR_INVALID, "n < 1");
  if (n > ((int64_t)1 << 32)) return set_error(GMS_ERR_TOO_LARGE, "autotune sizes are limited to 2^32 keys");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t kb = (size_t)n * (dtype >= 3 ? 8 : 4);
  const size_t vb = kv ? (size_t)n * 4 : 0;
  TuneBuffers b;  // 0 keys, 1 vals, 2 keys in (clobbered), 3 vals in, 4 keys out, 5 vals out, 6 first out, 7 flag
  size_t sizes[8] = {kb, vb, kb, vb, kb, vb, kb + vb, sizeof(int)};
  for (int i = 0; i < 8; ++i) {
    if (!sizes[i]) continue;
    cudaError_t e = cudaMalloc(&b.p[i], sizes[i]);
    if (e != cudaSuccess) return cuda_error(e, "autotune buffers");
  }
  for (int i = 0; i < 2; ++i) {
    cudaError_t e = cudaEventCreate(&b.ev[i]);
    if (e != cudaSuccess) return cuda_error(e, "autotune events");
  }
  fill_kernel<<<1024, 256, 0, st>>>(b.p[0], (int32_t*)b.p[1], n, dtype, 0x5eedull + (uint64_t)n);
  cudaMemsetAsync(b.p[7], 0, sizeof(int), st);

  // Candidates: fan-in, sample block and merge path.  With no merge round the
  // tuning has no effect and only the defaults are timed.
  std::vector<gms::Tune> cands;
  if (gms_rounds(dtype, kv, n) == 0) {
    cands.push_back(gms::Tune{});
  } else {
    for (int k : {32, 16, 8})
      for (int sb : {32, 16, 64})
        for (int bulk : {1, 3, 2, 0}) {
          if (!valid_tune(k, sb)) continue;
          gms::Tune t;
          t.k = k;
          t.sample_b = sb;
          t.bulk_copy = bulk;
          cands.push_back(t);
        }
  }
  const int was_timing = timing_suspend();
  struct Resume {
    int w;
    ~Resume() { timing_resume(w); }
  } resume{was_timing};

  double best_ms = 1e30;
  gms::Tune best;
  bool have_first = false;
  // stage 1: every candidate above; stage 2: the best one with the direct
  // (findPartitions-style) splitter instead of the sample-bracketed one;
  // stage 3: the other base case
  auto try_tune = [&](const gms::Tune& t) -> int {
    OverrideScope scope(&t);
    auto one = [&]() -> int {
      cudaMemcpyAsync(b.p[2], b.p[0], kb, cudaMemcpyDeviceToDevice, st);
      if (kv) cudaMemcpyAsync(b.p[3], b.p[1], vb, cudaMemcpyDeviceToDevice, st);
      cudaEventRecord(b.ev[0], st);
      const int rc = run_one(dtype, kv, b.p[2], (int32_t*)b.p[3], b.p[4], (int32_t*)b.p[5], n, st);
      cudaEventRecord(b.ev[1], st);
      return rc;
    };
    if (one() != GMS_OK) return GMS_OK;  // a tuning too fine for this n: not a candidate
    // Every tuning must give the same bits (the result of a sort is unique).
    if (!have_first) {
      cudaMemcpyAsync(b.p[6], b.p[4], kb, cudaMemcpyDeviceToDevice, st);
      if (kv) cudaMemcpyAsync((char*)b.p[6] + kb, b.p[5], vb, cudaMemcpyDeviceToDevice, st);
      have_first = true;
    } else {
      differ_kernel<<<1024, 256, 0, st>>>((const uint32_t*)b.p[6], (const uint32_t*)b.p[4], (int64_t)(kb / 4),
                                          (int*)b.p[7]);
      if (kv)
        differ_kernel<<<1024, 256, 0, st>>>((const uint32_t*)((char*)b.p[6] + kb), (const uint32_t*)b.p[5],
                                            (int64_t)(vb / 4), (int*)b.p[7]);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "autotune");
    float ms = 0;
    cudaEventElapsedTime(&ms, b.ev[0], b.ev[1]);
    // Repeats: enough for ~30 ms of sorting, at least 3; the median counts.
    const int reps = ms > 10.f ? 3 : (ms > 0.f ? std::min(25, std::max(3, (int)(30.f / ms))) : 3);
    std::vector<float> times;
    for (int r = 0; r < reps; ++r) {
      if (one() != GMS_OK) return GMS_ERR_INTERNAL;
      e = cudaEventSynchronize(b.ev[1]);
      if (e != cudaSuccess) return cuda_error(e, "autotune");
      cudaEventElapsedTime(&ms, b.ev[0], b.ev[1]);
      times.push_back(ms);
    }
    std::sort(times.begin(), times.end());
    const double med = times[times.size() / 2];
    if (med < best_ms) {
      best_ms = med;
      best = t;
    }
    return GMS_OK;
  };
  for (const gms::Tune& t : cands) {
    const int rc = try_tune(t);
    if (rc != GMS_OK) return rc;
  }
  if (have_first && gms_rounds(dtype, kv, n) > 0) {
    gms::Tune t2 = best;
    t2.split = 1;
    const int rc = try_tune(t2);
    if (rc != GMS_OK) return rc;
  }
  // stage 3 (keys-only sorts): the per-thread base case instead of the
  // warp-shuffle one, with the best tuning so far
  if (have_first && !kv) {
    gms::Tune t3 = best;
    t3.base = 1;
    const int rc = try_tune(t3);
    if (rc != GMS_OK) return rc;
  }
  if (!have_first) return set_error(GMS_ERR_INTERNAL, "no tuning candidate ran");
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, b.p[7], sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "autotune");
  if (flag) return set_error(GMS_ERR_INTERNAL, "tunings disagree on the sorted result");
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    table_put(dtype, kv, size_class(n), best, best_ms);
  }
  if (out_k) *out_k = best.k;
  if (out_sample_b) *out_sample_b = best.sample_b;
  if (out_bulk_copy) *out_bulk_copy = best.bulk_copy;
  if (out_ms) *out_ms = best_ms;
  return GMS_OK;
}

int gms_autotune_table(char* buf, size_t cap, size_t* needed) {
  clear_error();
  std::string s;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    s = table_json_locked();
  }
  if (needed) *needed = s.size() + 1;
  if (!buf || cap < s.size() + 1) return buf ? set_error(GMS_ERR_TOO_LARGE, "buffer too small") : GMS_OK;
  memcpy(buf, s.c_str(), s.size() + 1);
  return GMS_OK;
}

int gms_autotune_clear(void) {
  clear_error();
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_table.clear();
  return GMS_OK;
}

int gms_autotune_save(const char* path) {
  clear_error();
  if (!path) return set_error(GMS_ERR_INVALID, "null path");
  std::string dev;
  int status = device_name(&dev);
  if (status != GMS_OK) return status;
  std::string body;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    body = table_json_locked();
  }
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) return set_error(GMS_ERR_INVALID, "tune cache: cannot write file");
  f << "{\"format\": \"gms-tune-1\", \"device\": \"" << json_escape(dev) << "\", \"entries\": " << body << "}\n";
  return f.good() ? GMS_OK : set_error(GMS_ERR_INVALID, "tune cache: write failed");
}

int gms_autotune_load(const char* path) {
  clear_error();
  if (!path) return set_error(GMS_ERR_INVALID, "null path");
  return load_cache(path);
}

}  // extern "C"
