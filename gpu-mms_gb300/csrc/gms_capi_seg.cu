// C ABI: host side of the batched (segmented) sorts, and CUDA-graph capture of
// a sort.  The batched entry points themselves sit with the plain sorts of
// their key type (gms_capi_k32.cu, gms_capi_k64.cu, gms_capi_kv.cu), whose
// kernels they share.
#include <algorithm>
#include <new>
#include <vector>

#include "gms_capi_seg.cuh"

using namespace gms_capi;

namespace gms_capi {

int read_offsets(const int64_t* off, int64_t nseg, int64_t n, cudaStream_t st, std::vector<int64_t>* h) {
  h->assign((size_t)nseg + 1, 0);
  cudaError_t e = cudaMemcpyAsync(h->data(), off, sizeof(int64_t) * (size_t)(nseg + 1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "reading the offsets");
  const std::vector<int64_t>& o = *h;
  if (o[0] != 0 || o[(size_t)nseg] != n) return set_error(GMS_ERR_INVALID, "offsets must start at 0 and end at n");
  for (int64_t s = 0; s < nseg; ++s) {
    if (o[(size_t)s + 1] < o[(size_t)s]) return set_error(GMS_ERR_INVALID, "offsets must not decrease");
  }
  return GMS_OK;
}

int seg_upload(SegJob* job, void* dblob, cudaStream_t st) {
  std::vector<unsigned char> host(job->blob.bytes);
  gms::seg_blob_fill(job->plan, job->blob, host.data());
  // from pageable memory: the call returns once the bytes are staged, so the
  // host buffer may go right after it
  const cudaError_t e = cudaMemcpyAsync(dblob, host.data(), job->blob.bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_error(e, "uploading the batch plan");
  gms::seg_bind(job->plan, job->blob, dblob, &job->dev);
  return GMS_OK;
}

}  // namespace gms_capi

// ---------------------------------------------------------------------------
// CUDA graphs
struct gms_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> owned;        // device buffers the captured launches use
  gms_capi::SegJob* job = nullptr;  // plan of a captured batched sort
};

namespace {

template <class F>
int capture(cudaStream_t st, gms_graph** out, F&& body) {
  if (!out) return set_error(GMS_ERR_INVALID, "null graph handle");
  *out = nullptr;
  // 1. run once outside capture: sets kernel attributes, sizes the scratch
  int status = body();
  if (status != GMS_OK) return status;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamSynchronize");
  // 2. capture the same launch sequence
  const int was_timing = timing_suspend();
  e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    timing_resume(was_timing);
    return cuda_error(e, "cudaStreamBeginCapture");
  }
  status = body();
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  timing_resume(was_timing);
  if (status != GMS_OK) {
    if (g) cudaGraphDestroy(g);
    return status;
  }
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_error(e, "cudaGraphInstantiate");
  }
  gms_graph* h = new (std::nothrow) gms_graph;
  if (!h) {
    cudaGraphExecDestroy(x);
    cudaGraphDestroy(g);
    return set_error(GMS_ERR_NOMEM, "graph handle");
  }
  h->graph = g;
  h->exec = x;
  *out = h;
  return GMS_OK;
}

}  // namespace

extern "C" {

int gms_graph_create_sort_i32(int32_t* in, int32_t* out, int64_t n, void* stream, gms_graph** graph) {
  clear_error();
  cudaStream_t st = (cudaStream_t)stream;
  if (!st) return set_error(GMS_ERR_INVALID, "graph capture needs a non-default stream");
  return capture(st, graph, [&]() { return gms_sort_i32(in, out, n, 0, stream); });
}

int gms_graph_create_segmented_i32(int32_t* in, int32_t* out, int64_t n, const int64_t* offsets, int64_t nseg,
                                   void* stream, gms_graph** graph) {
  clear_error();
  cudaStream_t st = (cudaStream_t)stream;
  if (!st) return set_error(GMS_ERR_INVALID, "graph capture needs a non-default stream");
  if (!graph) return set_error(GMS_ERR_INVALID, "null graph handle");
  *graph = nullptr;
  if (n <= 0 || nseg <= 0 || !in || !out || !offsets) return set_error(GMS_ERR_INVALID, "empty batch or null pointer");
  // The plan, its device arrays, the scratch and the scratch array of n keys
  // belong to the graph (not to the per-stream cache, whose buffers a later
  // call may regrow), so the captured launches stay valid until it is destroyed.
  std::vector<int64_t> h;
  int status = read_offsets(offsets, nseg, n, st, &h);
  if (status != GMS_OK) return status;
  int64_t longest = 0;
  for (int64_t s = 0; s < nseg; ++s) longest = std::max(longest, h[(size_t)(s + 1)] - h[(size_t)s]);
  const gms::Tune t = tune_for_batch(0, 0, n, longest);
  SegJob* job = new (std::nothrow) SegJob;
  if (!job) return set_error(GMS_ERR_NOMEM, "graph plan");
  status = seg_prepare_i32(h, nseg, t, job);
  void* blob = nullptr;
  void* ws = nullptr;
  void* tmp = nullptr;
  auto fail = [&](int st2) {
    cudaFree(blob);
    cudaFree(ws);
    cudaFree(tmp);
    delete job;
    return st2;
  };
  if (status != GMS_OK) return fail(status);
  cudaError_t e = cudaMalloc(&blob, job->blob.bytes);
  if (e == cudaSuccess) e = cudaMalloc(&ws, job->ws_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&tmp, sizeof(uint32_t) * (size_t)n);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws, 0, 256, st);
  if (e != cudaSuccess) return fail(cuda_error(e, "graph buffers"));
  status = seg_upload(job, blob, st);
  if (status != GMS_OK) return fail(status);
  status = capture(st, graph, [&]() {
    const cudaError_t ee = seg_sort_i32(*job, ws, in, (int32_t*)tmp, out, n, t, st);
    return ee == cudaSuccess ? GMS_OK : cuda_error(ee, "segmented sort");
  });
  if (status != GMS_OK) return fail(status);
  (*graph)->owned = {blob, ws, tmp};
  (*graph)->job = job;
  return GMS_OK;
}

int gms_graph_launch(gms_graph* graph, void* stream) {
  clear_error();
  if (!graph || !graph->exec) return set_error(GMS_ERR_INVALID, "null graph");
  cudaError_t e = cudaGraphLaunch(graph->exec, (cudaStream_t)stream);
  return e == cudaSuccess ? GMS_OK : cuda_error(e, "cudaGraphLaunch");
}

int gms_graph_destroy(gms_graph* graph) {
  clear_error();
  if (!graph) return GMS_OK;
  if (graph->exec) cudaGraphExecDestroy(graph->exec);
  if (graph->graph) cudaGraphDestroy(graph->graph);
  for (void* p : graph->owned) cudaFree(p);
  delete graph->job;
  delete graph;
  return GMS_OK;
}

}  // extern "C"
