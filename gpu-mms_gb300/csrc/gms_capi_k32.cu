// C ABI: 32-bit keys (int32, uint32, float32), keys only.
#include <algorithm>
#include <mutex>
#include <vector>

#include "gms_capi.cuh"
#include "gms_capi_seg.cuh"

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

// ---- host-to-host sorts: copy in, sort, copy out, pipelined ----
//
// Per (device, stream): an input-copy stream and an output-copy stream, and
// kSlots slots of device buffers (input/scratch and output).  Asynchronous
// calls take the slots in turn, so that the input copy of call i+1 and the
// output copy of call i-1 overlap the sort of call i, and a slot waits only
// for the output copy of the call kSlots back; a synchronous call drains
// before it returns and always takes slot 0.  A slot's buffers are allocated
// when it is first used.  Within one call the input arrives in up to kChunks
// pieces and the base case sorts each piece's tiles as soon as it lands.
constexpr int kSlots = 3;
constexpr int kChunks = gms::kHostChunks;
constexpr int kOutParts = 8;  // parts of the last merge round

struct HostPipe {
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaStream_t side[2] = {nullptr, nullptr};  // chunk streams of a synchronous call's early rounds
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[2] = {nullptr, nullptr};
  void* din[kSlots] = {};
  void* dout[kSlots] = {};
  size_t cap[kSlots] = {};
  cudaEvent_t ready[kSlots][kChunks];
  int64_t start[kSlots][kChunks + 1];  // chunk boundaries in base tiles
  cudaEvent_t part[kSlots][kOutParts];
  cudaEvent_t sorted[kSlots];
  cudaEvent_t drained[kSlots];
  bool used[kSlots] = {};
  uint64_t async_calls = 0;
};

std::mutex g_pipe_mu;
std::vector<HostPipe*> g_pipes;

// Copies out the final prefix of the output after each part of the last
// round: records an event on the sort stream, and the output-copy stream
// waits for it before copying [done, safe).
struct OutDrain {
  HostPipe* p;
  int slot;
  int32_t* host_out;
  const int32_t* dev_out;
  int64_t done;
  cudaError_t err;
  int used = 0;
  static void after_part(void* ctx, int64_t safe, cudaStream_t st) {
    OutDrain* d = static_cast<OutDrain*>(ctx);
    if (d->err != cudaSuccess || safe <= d->done || d->used >= kOutParts) return;
    cudaEvent_t ev = d->p->part[d->slot][d->used++];
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(d->p->d2h, ev, 0);
    gms::hook_before(gms::KC_D2H, d->p->d2h);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d->host_out + d->done, d->dev_out + d->done, sizeof(int32_t) * (size_t)(safe - d->done),
                          cudaMemcpyDeviceToHost, d->p->d2h);
    gms::hook_after(gms::KC_D2H, d->p->d2h);
    if (e == cudaSuccess) d->done = safe;
    d->err = e;
  }
};

int pipe_for(cudaStream_t st, HostPipe** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  for (HostPipe* p : g_pipes) {
    if (p->dev == dev && p->st == st) {
      *out = p;
      return GMS_OK;
    }
  }
  HostPipe* p = new HostPipe();
  p->dev = dev;
  p->st = st;
  e = cudaStreamCreateWithFlags(&p->h2d, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->d2h, cudaStreamNonBlocking);
  for (int j = 0; j < 2 && e == cudaSuccess; ++j) {
    e = cudaStreamCreateWithFlags(&p->side[j], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->join[j], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
  for (int s = 0; s < kSlots && e == cudaSuccess; ++s) {
    for (int c = 0; c < kChunks && e == cudaSuccess; ++c) e = cudaEventCreateWithFlags(&p->ready[s][c], cudaEventDisableTiming);
    for (int c = 0; c < kOutParts && e == cudaSuccess; ++c) e = cudaEventCreateWithFlags(&p->part[s][c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->sorted[s], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->drained[s], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    delete p;  // the few handles created before the failure stay allocated
    return cuda_error(e, "host pipeline setup");
  }
  g_pipes.push_back(p);
  *out = p;
  return GMS_OK;
}

// sync: the caller waits for this call before the next (slot 0), and the
// early merge rounds run piece by piece as the input lands (worth it when
// nothing else overlaps the copies; a pipeline of calls already overlaps them
// with the neighbouring sorts).
int host_sort_enqueue(const int32_t* host_in, int32_t* host_out, int64_t n, cudaStream_t st, bool sync) {
  clear_error();
  if (n < 0) return set_error(GMS_ERR_INVALID, "n < 0");
  if (n == 0) return GMS_OK;
  if (!host_in || !host_out) return set_error(GMS_ERR_INVALID, "null pointer");
  std::lock_guard<std::mutex> g(g_pipe_mu);
  HostPipe* p = nullptr;
  int status = pipe_for(st, &p);
  if (status != GMS_OK) return status;
  const size_t bytes = sizeof(int32_t) * (size_t)n;
  cudaError_t e = cudaSuccess;
  const int slot = sync ? 0 : (int)(p->async_calls++ % kSlots);
  if (bytes > p->cap[slot]) {
    // growing: wait for the slot's last call (its output copy ends it), then
    // reallocate the slot
    if (p->used[slot]) e = cudaEventSynchronize(p->drained[slot]);
    if (e != cudaSuccess) return cuda_error(e, "host pipeline drain");
    cudaFree(p->din[slot]);
    cudaFree(p->dout[slot]);
    p->din[slot] = p->dout[slot] = nullptr;
    p->cap[slot] = 0;
    e = cudaMalloc(&p->din[slot], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&p->dout[slot], bytes);
    if (e != cudaSuccess) return cuda_error(e, "host pipeline buffers");
    p->cap[slot] = bytes;
  }
  // the slot's previous call must have drained its output before reuse
  if (p->used[slot]) {
    e = cudaStreamWaitEvent(p->h2d, p->drained[slot], 0);
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamWaitEvent");
  }
  // Up to kChunks pieces of whole base tiles (host_chunk_plan), the first one small
  // so that the sort starts soon after the call.
  const gms::Tune tune = tune_for(0, 0, n);
  const int64_t bt = EngI32::base_tile(tune);
  const int64_t tiles = gms::ceil_div(n, bt);
  int64_t* start = p->start[slot];
  gms::BaseGate gate;
  gate.chunks = gms::host_chunk_plan(tiles, tune.k, EngI32::passes_for(n, tune), start);
  gate.start = start;
  gate.ready = p->ready[slot];
  gate.early_rounds = sync;
  if (sync) {
    // chunks alternate between two streams so that one chunk's small sample
    // merges and splitters overlap the next chunk's base case and merges
    gate.side = p->side;
    gate.fork = p->fork;
    gate.join = p->join;
  }
  for (int c = 0; c < gate.chunks; ++c) {
    const int64_t k0 = std::min(n, start[c] * bt);
    const int64_t k1 = std::min(n, start[c + 1] * bt);
    if (k1 > k0) {
      gms::hook_before(gms::KC_H2D, p->h2d);
      e = cudaMemcpyAsync((int32_t*)p->din[slot] + k0, host_in + k0, sizeof(int32_t) * (size_t)(k1 - k0),
                          cudaMemcpyHostToDevice, p->h2d);
      gms::hook_after(gms::KC_H2D, p->h2d);
      if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync H2D");
    }
    e = cudaEventRecord(p->ready[slot][c], p->h2d);
    if (e != cudaSuccess) return cuda_error(e, "cudaEventRecord");
  }
  // Output copy: the last merge round runs in parts, and after each part the
  // keys known to be final (a prefix of the output) are copied out while the
  // next part merges; the rest follows the sort.
  OutDrain drain{p, slot, host_out, (const int32_t*)p->dout[slot], 0, cudaSuccess};
  gms::RoundSplit split;
  split.parts = kOutParts;
  split.ramp = true;
  split.after = &OutDrain::after_part;
  split.ctx = &drain;
  status = run_sort<EngI32, uint32_t, NoVal>((uint32_t*)p->din[slot], nullptr, (uint32_t*)p->dout[slot], nullptr, n, st,
                                             0, nullptr, 0, &gate, &split);
  if (status != GMS_OK) return status;
  if (drain.err != cudaSuccess) return cuda_error(drain.err, "host pipeline output");
  e = cudaEventRecord(p->sorted[slot], st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(p->d2h, p->sorted[slot], 0);
  if (e == cudaSuccess && drain.done < n) {
    gms::hook_before(gms::KC_D2H, p->d2h);
    e = cudaMemcpyAsync(host_out + drain.done, (const int32_t*)p->dout[slot] + drain.done,
                        sizeof(int32_t) * (size_t)(n - drain.done), cudaMemcpyDeviceToHost, p->d2h);
    gms::hook_after(gms::KC_D2H, p->d2h);
  }
  if (e == cudaSuccess) e = cudaEventRecord(p->drained[slot], p->d2h);
  if (e != cudaSuccess) return cuda_error(e, "host pipeline output");
  p->used[slot] = true;
  return GMS_OK;
}

int host_sync(cudaStream_t st) {
  clear_error();
  std::lock_guard<std::mutex> g(g_pipe_mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  for (HostPipe* p : g_pipes) {
    if (p->dev == dev && p->st == st) {
      e = cudaStreamSynchronize(p->h2d);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(p->d2h);
      if (e != cudaSuccess) return cuda_error(e, "host pipeline sync");
      return GMS_OK;
    }
  }
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "cudaStreamSynchronize");
}

}  // namespace

void gms_capi::release_host_pipes() {
  std::lock_guard<std::mutex> g(g_pipe_mu);
  for (HostPipe* p : g_pipes) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(p->dev);
    cudaStreamSynchronize(p->h2d);
    cudaStreamSynchronize(p->d2h);
    for (int s = 0; s < kSlots; ++s) {
      cudaFree(p->din[s]);
      cudaFree(p->dout[s]);
      for (int c = 0; c < kChunks; ++c) cudaEventDestroy(p->ready[s][c]);
      for (int c = 0; c < kOutParts; ++c) cudaEventDestroy(p->part[s][c]);
      cudaEventDestroy(p->sorted[s]);
      cudaEventDestroy(p->drained[s]);
    }
    for (int j = 0; j < 2; ++j) {
      cudaStreamSynchronize(p->side[j]);
      cudaStreamDestroy(p->side[j]);
      cudaEventDestroy(p->join[j]);
    }
    cudaEventDestroy(p->fork);
    cudaStreamDestroy(p->h2d);
    cudaStreamDestroy(p->d2h);
    cudaSetDevice(cur);
    delete p;
  }
  g_pipes.clear();
}

int gms_capi::seg_prepare_i32(const std::vector<int64_t>& off, int64_t nseg, const gms::Tune& t, SegJob* job) {
  return seg_prepare<EngI32, uint32_t>(off, nseg, t, job);
}

cudaError_t gms_capi::seg_sort_i32(const SegJob& job, void* ws, const int32_t* in, int32_t* tmp, int32_t* out,
                                   int64_t n, const gms::Tune& t, cudaStream_t st) {
  const gms::WsPtrs<uint32_t> w = gms::ws_carve<uint32_t>(gms::seg_ws_layout(job.plan), t.k, ws);
  return EngI32::seg_sort(w, job.dev, (const uint32_t*)in, nullptr, (uint32_t*)tmp, nullptr, (uint32_t*)out, nullptr,
                          n, t, st);
}

int gms_capi::seg_run_i32(SegJob* job, const void* dblob, const int32_t* in, int32_t* out, int64_t n,
                          const gms::Tune& t, cudaStream_t st) {
  return run_planned<EngI32, uint32_t, NoVal>(job, dblob, (const uint32_t*)in, nullptr, (uint32_t*)out, nullptr, n, t,
                                              st);
}

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
    const gms::WsLayout l = EngI32::plan_merge_level<uint32_t>(task_size, size, t);
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

int gms_sort_host_i32_async(const int32_t* host_in, int32_t* host_out, int64_t n, void* stv) {
  return host_sort_enqueue(host_in, host_out, n, (cudaStream_t)stv, false);
}

int gms_host_sync(void* stv) { return host_sync((cudaStream_t)stv); }

int gms_sort_host_i32(const int32_t* host_in, int32_t* host_out, int64_t n, void* stv) {
  const int status = host_sort_enqueue(host_in, host_out, n, (cudaStream_t)stv, true);
  if (status != GMS_OK) return status;
  return host_sync((cudaStream_t)stv);
}

int gms_segmented_sort_i32(const int32_t* in, int32_t* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<EngI32, uint32_t, NoVal>((const uint32_t*)in, nullptr, (uint32_t*)out, nullptr, n, offsets, nseg,
                                                (cudaStream_t)st, 0);
}
int gms_segmented_sort_u32(const uint32_t* in, uint32_t* out, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* st) {
  return run_segmented<EngU32, uint32_t, NoVal>(in, nullptr, out, nullptr, n, offsets, nseg, (cudaStream_t)st, 1);
}
int gms_segmented_sort_f32(const float* in, float* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return run_segmented<EngF32, uint32_t, NoVal>((const uint32_t*)in, nullptr, (uint32_t*)out, nullptr, n, offsets, nseg,
                                                (cudaStream_t)st, 2);
}

}  // extern "C"
