// C ABI: batched (segmented) sorts and CUDA-graph capture of a sort.
#include <new>

#include "gms_capi.cuh"
#include "gms_segmented.cuh"

using namespace gms_capi;

namespace {

using CompEngine = KeysEngine<uint64_t, gms::IdentityCodec<uint64_t>>;

// Flags the status word if the offsets are not 0 = off[0] <= ... <= off[nseg] = n.
__global__ void check_offsets_kernel(const int64_t* __restrict__ off, int64_t nseg, int64_t n, int* err) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += stride) {
    const bool bad = off[s] > off[s + 1] || (s == 0 && off[0] != 0) || (s == nseg - 1 && off[nseg] != n);
    if (bad && err) atomicOr(err, 8);
  }
}

template <class Codec32>
int segmented32(void* in, void* out, int64_t n, const int64_t* off, int64_t nseg, cudaStream_t st) {
  clear_error();
  if (n < 0 || nseg < 0) return set_error(GMS_ERR_INVALID, "n < 0 or nseg < 0");
  if (n == 0 || nseg == 0) return GMS_OK;
  if (!in || !out || !off) return set_error(GMS_ERR_INVALID, "null pointer");
  if (nseg > 0xffffffffll) return set_error(GMS_ERR_TOO_LARGE, "more than 2^32 segments");
  if (n > ((int64_t)1 << 37)) return set_error(GMS_ERR_TOO_LARGE, "n beyond 2^37");
  const gms::Tune t = tune_for(4, 0, n);  // the composites sort as uint64 keys
  const gms::WsLayout l = CompEngine::plan(n, t);
  if (!l.ok) return set_error(GMS_ERR_INVALID, "tuning too fine for this n (sample recursion too deep)");
  int status = GMS_OK;
  void* ws = cache_get(0, gms::ws_bytes_for<uint64_t>(l, t.k), st, &status);
  if (status != GMS_OK) return status;
  const gms::WsPtrs<uint64_t> w = gms::ws_carve<uint64_t>(l, t.k, ws);
  uint64_t* ca = (uint64_t*)cache_get(30, sizeof(uint64_t) * (size_t)n, st, &status);
  if (status != GMS_OK) return status;
  uint64_t* cb = (uint64_t*)cache_get(31, sizeof(uint64_t) * (size_t)n, st, &status);
  if (status != GMS_OK) return status;
  check_offsets_kernel<<<(unsigned)gms::ceil_div(nseg, 256) > 4096 ? 4096 : (unsigned)gms::ceil_div(nseg, 256), 256, 0,
                         st>>>(off, nseg, n, w.err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "check_offsets_kernel");
  gms::build_composite_kernel<Codec32>
      <<<(unsigned)gms::ceil_div(n, gms::kSegChunk), gms::kSegThreads, 0, st>>>((const uint32_t*)in, off, nseg, n, ca);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "build_composite_kernel");
  e = CompEngine::sort(w, ca, nullptr, cb, nullptr, n, t, st);
  if (e != cudaSuccess) return cuda_error(e, "segmented sort");
  const int64_t blocks = gms::ceil_div(n, 1024) < 65536 ? gms::ceil_div(n, 1024) : 65536;
  gms::extract_composite_kernel<Codec32><<<(unsigned)blocks, 256, 0, st>>>(cb, (uint32_t*)out, n);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "extract_composite_kernel");
  return GMS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// CUDA graphs
struct gms_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
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

int gms_segmented_sort_i32(int32_t* in, int32_t* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return segmented32<gms::SignFlip32>(in, out, n, offsets, nseg, (cudaStream_t)st);
}
int gms_segmented_sort_u32(uint32_t* in, uint32_t* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return segmented32<gms::IdentityCodec<uint32_t>>(in, out, n, offsets, nseg, (cudaStream_t)st);
}
int gms_segmented_sort_f32(float* in, float* out, int64_t n, const int64_t* offsets, int64_t nseg, void* st) {
  return segmented32<gms::FloatOrder32>(in, out, n, offsets, nseg, (cudaStream_t)st);
}

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
  return capture(st, graph, [&]() { return gms_segmented_sort_i32(in, out, n, offsets, nseg, stream); });
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
  delete graph;
  return GMS_OK;
}

}  // extern "C"
