// Continuous-batching sort server (C ABI: gms_server_*).
//
// No counterpart in the reference, which is a synchronous one-call-per-array
// library (GPU-MMS src/multimergesort.hxx:56-141, cudaDeviceSynchronize at 137).
//
// Requests are device-resident key buffers (int32 keys, or uint64 keys with an
// int32 payload); results go to caller-owned device output buffers; inputs are
// never modified.  A dispatcher thread turns queued requests into work items:
//   * requests of one kind of at most `batch_max_keys` keys that are waiting
//     together become ONE batched sort (a segmented sort planned on the host
//     from the requests' sizes, its plan uploaded from pinned memory, so the
//     dispatcher never waits for a stream);
//   * larger requests run one per item.
// Each item is admitted only when its device memory (staging buffers,
// allocated stream-ordered with cudaMallocAsync so no allocation stalls other
// streams, plus the sort scratch of its stream) fits the memory budget still
// free; items are spread over a pool of streams so several run on the device
// at once, and new requests keep being admitted while earlier ones run.  A
// completion thread waits on each item's event, frees its staging memory,
// stamps the completion time of its requests and returns their budget.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "gms_capi.cuh"
#include "gms_capi_seg.cuh"

using namespace gms_capi;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id;
  int kind;  // 0: int32 keys; 1: uint64 keys + int32 payload
  const void* kin;
  const int32_t* vin;
  void* kout;
  int32_t* vout;
  int64_t n;
  Clock::time_point t_submit;
  Clock::time_point t_done;
  bool done = false;
  int status = GMS_OK;
};

struct Item {
  std::vector<uint64_t> reqs;
  int stream_idx = 0;
  cudaEvent_t ev = nullptr;
  size_t bytes = 0;         // budget charged
  std::vector<void*> bufs;  // stream-ordered allocations to release
  // batched items: the plan, its tuning, and the pinned slot its arrays are
  // uploaded from (free again once the item's event completes)
  std::unique_ptr<SegJob> job;
  gms::Tune tune;
  int pin_slot = -1;
};

// pinned upload slot of a batch plan
constexpr size_t kPinSlotBytes = size_t(1) << 20;

}  // namespace

struct gms_server {
  int device = 0;
  size_t budget = 0;
  size_t in_use = 0;
  int64_t batch_max_keys = 0;
  int64_t batch_cap_keys = 0;
  std::vector<cudaStream_t> streams;
  int next_stream = 0;

  std::mutex mu;
  std::condition_variable cv_queue;   // dispatcher: new requests / stop
  std::condition_variable cv_budget;  // dispatcher: memory freed
  std::condition_variable cv_done;    // waiters: a request finished
  std::deque<uint64_t> queue;
  std::map<uint64_t, Request> reqs;
  std::deque<Item> inflight;
  std::condition_variable cv_inflight;
  uint64_t next_id = 1;
  bool stop = false;
  int fatal = GMS_OK;
  std::string fatal_msg;
  std::vector<double> latencies_ms;
  int64_t keys_done = 0;
  Clock::time_point t_first, t_last;
  bool have_first = false;

  std::thread dispatcher, completer;
  unsigned char* pin = nullptr;  // pinned slots of batch plans
  std::vector<char> pin_free;
};

namespace {

size_t scratch_bytes_i32(int64_t n) { return gms_workspace_bytes(0, 0, n); }

// Device memory one item needs beyond its stream's reserved scratch.
size_t item_bytes(gms_server* s, const std::vector<uint64_t>& ids, bool batch, size_t plan_bytes) {
  int64_t n = 0;
  int kind = 0;
  for (uint64_t id : ids) {
    n += s->reqs[id].n;
    kind = s->reqs[id].kind;
  }
  const size_t elt = kind == 0 ? 4 : 8 + 4;
  if (batch) return (size_t)n * elt * 2 + plan_bytes + 4096;  // gathered in/out, the plan
  return (size_t)n * elt + 512;                               // staging copy of the input
}

void fail(gms_server* s, int status, const char* msg) {
  if (s->fatal == GMS_OK) {
    s->fatal = status;
    s->fatal_msg = msg;
  }
}

// Launches one item on its stream; called by the dispatcher without the lock.
int launch_item(gms_server* s, Item& it, const std::vector<Request*>& rs, bool batch) {
  cudaStream_t st = s->streams[it.stream_idx];
  cudaError_t e;
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    e = cudaMallocAsync(&p, bytes > 0 ? bytes : 16, st);
    if (e != cudaSuccess) return nullptr;
    it.bufs.push_back(p);
    return p;
  };
  if (batch) {
    const bool kvb = rs[0]->kind == 1;
    const size_t kb = kvb ? sizeof(uint64_t) : sizeof(int32_t);
    std::vector<int64_t> off(rs.size() + 1, 0);
    for (size_t i = 0; i < rs.size(); ++i) off[i + 1] = off[i] + rs[i]->n;
    const int64_t n = off.back();
    SegJob* job = it.job.get();
    unsigned char* bin = (unsigned char*)alloc(kb * n);
    unsigned char* bout = bin ? (unsigned char*)alloc(kb * n) : nullptr;
    int32_t* vbin = (bout && kvb) ? (int32_t*)alloc(sizeof(int32_t) * n) : nullptr;
    int32_t* vbout = vbin ? (int32_t*)alloc(sizeof(int32_t) * n) : nullptr;
    void* dblob = (bout && (!kvb || vbout)) ? alloc(job->blob.bytes) : nullptr;
    if (!dblob) return cuda_error(e, "cudaMallocAsync(batch)");
    // the plan's arrays, from the item's pinned slot (an asynchronous copy)
    unsigned char* slot = s->pin + (size_t)it.pin_slot * kPinSlotBytes;
    gms::seg_blob_fill(job->plan, job->blob, slot);
    e = cudaMemcpyAsync(dblob, slot, job->blob.bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "plan H2D");
    for (size_t i = 0; i < rs.size(); ++i) {
      e = cudaMemcpyAsync(bin + kb * off[i], rs[i]->kin, kb * rs[i]->n, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess && kvb)
        e = cudaMemcpyAsync(vbin + off[i], rs[i]->vin, sizeof(int32_t) * rs[i]->n, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_error(e, "gather D2D");
    }
    const int status = kvb ? seg_run_kv_u64(job, dblob, (const uint64_t*)bin, vbin, (uint64_t*)bout, vbout, n,
                                            it.tune, st)
                           : seg_run_i32(job, dblob, (const int32_t*)bin, (int32_t*)bout, n, it.tune, st);
    if (status != GMS_OK) return status;
    for (size_t i = 0; i < rs.size(); ++i) {
      e = cudaMemcpyAsync(rs[i]->kout, bout + kb * off[i], kb * rs[i]->n, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess && kvb)
        e = cudaMemcpyAsync(rs[i]->vout, vbout + off[i], sizeof(int32_t) * rs[i]->n, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_error(e, "scatter D2D");
    }
  } else {
    Request* r = rs[0];
    if (r->kind == 0) {
      int32_t* tmp = (int32_t*)alloc(sizeof(int32_t) * r->n);
      if (!tmp) return cuda_error(e, "cudaMallocAsync(i32)");
      e = cudaMemcpyAsync(tmp, r->kin, sizeof(int32_t) * r->n, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_error(e, "copy D2D");
      int status = gms_sort_i32(tmp, (int32_t*)r->kout, r->n, 0, st);
      if (status != GMS_OK) return status;
    } else {
      uint64_t* tk = (uint64_t*)alloc(sizeof(uint64_t) * r->n);
      int32_t* tv = tk ? (int32_t*)alloc(sizeof(int32_t) * r->n) : nullptr;
      if (!tv) return cuda_error(e, "cudaMallocAsync(kv)");
      e = cudaMemcpyAsync(tk, r->kin, sizeof(uint64_t) * r->n, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(tv, r->vin, sizeof(int32_t) * r->n, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_error(e, "copy D2D");
      int status = gms_sort_kv_u64_i32(tk, tv, (uint64_t*)r->kout, r->vout, r->n, 0, st);
      if (status != GMS_OK) return status;
    }
  }
  for (void* p : it.bufs) cudaFreeAsync(p, st);
  it.bufs.clear();
  e = cudaEventRecord(it.ev, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaEventRecord");
  return GMS_OK;
}

void dispatcher_main(gms_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv_queue.wait(lk, [&] { return s->stop || !s->queue.empty(); });
    if (s->stop && s->queue.empty()) break;
    // form one work item from the head of the queue
    std::vector<uint64_t> ids;
    bool batch = false;
    const uint64_t head = s->queue.front();
    const Request& h = s->reqs[head];
    if (h.n <= s->batch_max_keys) {
      // every small request of the head's kind waiting now joins the batch (up
      // to the cap)
      int64_t tot = 0;
      for (auto it = s->queue.begin(); it != s->queue.end();) {
        const Request& r = s->reqs[*it];
        if (r.kind == h.kind && r.n <= s->batch_max_keys && tot + r.n <= s->batch_cap_keys) {
          ids.push_back(*it);
          tot += r.n;
          it = s->queue.erase(it);
        } else {
          ++it;
        }
      }
      batch = true;
    } else {
      ids.push_back(head);
      s->queue.pop_front();
    }
    Item it;
    it.reqs = ids;
    size_t plan_bytes = 0;
    if (batch) {
      // plan the batch from its sizes, here on the host
      std::vector<int64_t> off(ids.size() + 1, 0);
      int64_t longest = 0;
      for (size_t i = 0; i < ids.size(); ++i) {
        off[i + 1] = off[i] + s->reqs[ids[i]].n;
        longest = std::max(longest, s->reqs[ids[i]].n);
      }
      const int kind = s->reqs[ids[0]].kind;
      it.tune = tune_for_batch(kind == 0 ? 0 : 4, kind, off.back(), longest);
      it.job.reset(new (std::nothrow) SegJob);
      int st2 = it.job ? (kind == 0 ? seg_prepare_i32(off, (int64_t)ids.size(), it.tune, it.job.get())
                                    : seg_prepare_kv_u64(off, (int64_t)ids.size(), it.tune, it.job.get()))
                       : GMS_ERR_NOMEM;
      if (st2 == GMS_OK && it.job->blob.bytes > kPinSlotBytes) st2 = GMS_ERR_TOO_LARGE;
      if (st2 != GMS_OK) {
        for (uint64_t id : ids) {
          Request& r = s->reqs[id];
          r.status = st2;
          r.done = true;
          r.t_done = Clock::now();
        }
        s->cv_done.notify_all();
        continue;
      }
      plan_bytes = it.job->blob.bytes;
    }
    it.bytes = item_bytes(s, ids, batch, plan_bytes);
    // admission: wait until the item fits the budget that is still free
    if (it.bytes > s->budget) {
      for (uint64_t id : ids) {
        Request& r = s->reqs[id];
        r.status = GMS_ERR_TOO_LARGE;
        r.done = true;
        r.t_done = Clock::now();
      }
      s->cv_done.notify_all();
      continue;
    }
    s->cv_budget.wait(lk, [&] { return s->stop || s->in_use + it.bytes <= s->budget; });
    if (batch) {
      // a free pinned slot for the plan upload (freed by the completer)
      auto free_slot = [&] {
        for (size_t i = 0; i < s->pin_free.size(); ++i)
          if (s->pin_free[i]) return (int)i;
        return -1;
      };
      s->cv_budget.wait(lk, [&] { return s->stop || free_slot() >= 0; });
      it.pin_slot = free_slot();
      if (it.pin_slot < 0) it.pin_slot = 0;  // stopping: the item still runs to completion
      s->pin_free[(size_t)it.pin_slot] = 0;
    }
    s->in_use += it.bytes;
    it.stream_idx = s->next_stream;
    s->next_stream = (s->next_stream + 1) % (int)s->streams.size();
    std::vector<Request*> rs;
    for (uint64_t id : ids) rs.push_back(&s->reqs[id]);
    lk.unlock();
    cudaEventCreateWithFlags(&it.ev, cudaEventDisableTiming);
    const int status = launch_item(s, it, rs, batch);
    lk.lock();
    if (status != GMS_OK) {
      fail(s, status, gms_last_error());
      for (void* p : it.bufs) cudaFreeAsync(p, s->streams[it.stream_idx]);
      it.bufs.clear();
      cudaEventRecord(it.ev, s->streams[it.stream_idx]);
      for (Request* r : rs) r->status = status;
    }
    s->inflight.push_back(std::move(it));
    s->cv_inflight.notify_all();
  }
  s->cv_inflight.notify_all();
}

void completer_main(gms_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv_inflight.wait(lk, [&] { return !s->inflight.empty() || (s->stop && s->queue.empty()); });
    if (s->inflight.empty()) {
      if (s->stop && s->queue.empty()) break;
      continue;
    }
    Item it = std::move(s->inflight.front());
    s->inflight.pop_front();
    lk.unlock();
    // a bounded host wait is not needed: the event always completes (device
    // waits inside the kernels are themselves bounded)
    cudaError_t e = cudaEventSynchronize(it.ev);
    const Clock::time_point now = Clock::now();
    cudaEventDestroy(it.ev);
    lk.lock();
    if (e != cudaSuccess) fail(s, cuda_error(e, "item event"), gms_last_error());
    s->in_use -= it.bytes;
    if (it.pin_slot >= 0) s->pin_free[(size_t)it.pin_slot] = 1;
    for (uint64_t id : it.reqs) {
      Request& r = s->reqs[id];
      r.done = true;
      r.t_done = now;
      if (e != cudaSuccess) r.status = GMS_ERR_CUDA;
      if (r.status == GMS_OK) {
        s->latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r.t_submit).count());
        s->keys_done += r.n;
        s->t_last = now;
      }
    }
    s->cv_budget.notify_all();
    s->cv_done.notify_all();
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int gms_server_create(size_t memory_budget, int nstreams, int64_t batch_max_keys, int64_t max_request_keys,
                      gms_server** out) {
  clear_error();
  if (!out || nstreams < 1 || nstreams > 64 || batch_max_keys < 0 || max_request_keys < 1)
    return set_error(GMS_ERR_INVALID, "bad server parameters");
  *out = nullptr;
  gms_server* s = new (std::nothrow) gms_server;
  if (!s) return set_error(GMS_ERR_NOMEM, "server");
  cudaGetDevice(&s->device);
  s->budget = memory_budget;
  s->batch_max_keys = batch_max_keys;
  s->batch_cap_keys = batch_max_keys * 64 > max_request_keys ? batch_max_keys * 64 : max_request_keys;
  for (int i = 0; i < nstreams; ++i) {
    cudaStream_t st;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      delete s;
      return cuda_error(e, "cudaStreamCreate");
    }
    s->streams.push_back(st);
    // scratch of every stream sized once for the largest request or batch,
    // so no sort allocates while the server runs: the plain sorts' scratch
    // (with room for a batch plan's somewhat larger sample arrays) and the
    // batched sorts' scratch arrays of keys and payload
    const int64_t most = max_request_keys > s->batch_cap_keys ? max_request_keys : s->batch_cap_keys;
    const size_t ws = std::max(gms_workspace_bytes(0, 0, most), gms_workspace_bytes(4, 1, most));
    int status = GMS_OK;
    cache_get(0, ws + ws / 4 + (size_t(1) << 20), st, &status);
    if (status == GMS_OK) cache_get(30, sizeof(uint64_t) * (size_t)s->batch_cap_keys, st, &status);
    if (status == GMS_OK) cache_get(31, sizeof(int32_t) * (size_t)s->batch_cap_keys, st, &status);
    if (status != GMS_OK) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      delete s;
      return status;
    }
  }
  // pinned upload slots of batch plans, two per stream
  {
    const size_t nslots = 2 * s->streams.size();
    cudaError_t e = cudaMallocHost((void**)&s->pin, nslots * kPinSlotBytes);
    if (e != cudaSuccess) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      delete s;
      return cuda_error(e, "cudaMallocHost(plan slots)");
    }
    s->pin_free.assign(nslots, 1);
  }
  // keep freed stream-ordered staging memory mapped up to the budget
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
    uint64_t thr = memory_budget;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  s->dispatcher = std::thread(dispatcher_main, s);
  s->completer = std::thread(completer_main, s);
  *out = s;
  return GMS_OK;
}

int gms_server_submit(gms_server* s, int kind, const void* keys_in, const int32_t* vals_in, void* keys_out,
                      int32_t* vals_out, int64_t n, uint64_t* id_out) {
  clear_error();
  if (!s || !id_out || (kind != 0 && kind != 1) || n < 0 || (n > 0 && (!keys_in || !keys_out)) ||
      (kind == 1 && n > 0 && (!vals_in || !vals_out)))
    return set_error(GMS_ERR_INVALID, "bad request");
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return set_error(GMS_ERR_INVALID, "server stopped");
  Request r;
  r.id = s->next_id++;
  r.kind = kind;
  r.kin = keys_in;
  r.vin = vals_in;
  r.kout = keys_out;
  r.vout = vals_out;
  r.n = n;
  r.t_submit = Clock::now();
  if (!s->have_first) {
    s->have_first = true;
    s->t_first = r.t_submit;
  }
  *id_out = r.id;
  if (n == 0) {
    r.done = true;
    r.t_done = r.t_submit;
    s->reqs[r.id] = r;
    s->cv_done.notify_all();
    return GMS_OK;
  }
  s->reqs[r.id] = r;
  s->queue.push_back(r.id);
  s->cv_queue.notify_one();
  return GMS_OK;
}

int gms_server_wait(gms_server* s, uint64_t id, double* latency_ms) {
  clear_error();
  if (!s) return set_error(GMS_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto f = s->reqs.find(id);
  if (f == s->reqs.end()) return set_error(GMS_ERR_INVALID, "unknown request id");
  s->cv_done.wait(lk, [&] { return s->reqs[id].done; });
  const Request& r = s->reqs[id];
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
  const int st = r.status;
  s->reqs.erase(id);
  if (st != GMS_OK) return set_error(st, "request failed");
  return GMS_OK;
}

int gms_server_drain(gms_server* s) {
  clear_error();
  if (!s) return set_error(GMS_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv_done.wait(lk, [&] {
    if (!s->queue.empty() || !s->inflight.empty()) return false;
    for (auto& kv : s->reqs)
      if (!kv.second.done) return false;
    return true;
  });
  return s->fatal == GMS_OK ? GMS_OK : set_error(s->fatal, s->fatal_msg.c_str());
}

// stats: completed requests, p50/p99 latency (ms), keys/s over first submit .. last completion
int gms_server_stats(gms_server* s, int64_t* completed, double* p50_ms, double* p99_ms, double* keys_per_s) {
  clear_error();
  if (!s) return set_error(GMS_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> g(s->mu);
  if (completed) *completed = (int64_t)s->latencies_ms.size();
  if (p50_ms) *p50_ms = percentile(s->latencies_ms, 0.50);
  if (p99_ms) *p99_ms = percentile(s->latencies_ms, 0.99);
  if (keys_per_s) {
    const double sec = s->have_first ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0.0;
    *keys_per_s = sec > 0 ? (double)s->keys_done / sec : 0.0;
  }
  return GMS_OK;
}

int gms_server_destroy(gms_server* s) {
  clear_error();
  if (!s) return GMS_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_queue.notify_all();
  s->cv_budget.notify_all();
  s->cv_inflight.notify_all();
  s->dispatcher.join();
  {
    std::lock_guard<std::mutex> g(s->mu);
  }
  s->cv_inflight.notify_all();
  s->completer.join();
  for (cudaStream_t st : s->streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  cudaFreeHost(s->pin);
  delete s;
  return GMS_OK;
}

}  // extern "C"
