/*
 * gms.h -- C ABI of the GB300 multiway mergesort (libgms.so).
 *
 * Plain pointers and sizes only.  Every device pointer is a CUDA global-memory
 * pointer on the current device; `stream` is a cudaStream_t passed as void*
 * (NULL = legacy default stream).  Every call returns a gms_status (0 = OK) and
 * records a message readable with gms_last_error() on the calling thread.
 * Calls are asynchronous on `stream` unless stated otherwise.
 *
 * Each entry point names the GPU-MMS interface it replaces (paths relative to
 * the GPU-MMS source tree).
 */
#ifndef GMS_H_
#define GMS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gms_status {
  GMS_OK = 0,
  GMS_ERR_INVALID = 1,   /* bad argument: null pointer, negative size, bad fan-in ... */
  GMS_ERR_CUDA = 2,      /* a CUDA call failed; gms_last_error() has the CUDA message */
  GMS_ERR_NOMEM = 3,     /* device scratch could not be allocated                      */
  GMS_ERR_TOO_LARGE = 4, /* size beyond what this library supports                     */
  GMS_ERR_INTERNAL = 5
} gms_status;

/* Library version (major*10000 + minor*100 + patch). */
int gms_version(void);
/* Human-readable name of a status code. */
const char* gms_status_string(int status);
/* Last error message recorded on the calling thread ("" if none). */
const char* gms_last_error(void);

/* ---------------------------------------------------------------------------
 * Plain sorts.
 *
 * Replaces: template<typename T, fptr_t f> T* multimergesort(T* input,
 *   T* output, T* h_data, int N)            src/multimergesort.hxx:56-141
 * and the documented 5-argument form multimergesort<T,cmp>(input, output,
 *   host_array, threadBlocks, N)             README.md:16-25
 *
 * Sorts `n` keys ascending.  `input` and `output` are device arrays of n keys.
 * The sorted keys are ALWAYS in `output` (the reference returns whichever of
 * its two buffers holds the result; here that buffer is always `output`).
 * `input` is used as scratch and its contents are clobbered, as in the
 * reference.  `thread_blocks` is the reference's threadBlocks hint: <= 0 lets
 * the library choose; a positive value is accepted and recorded (the grids of
 * this implementation are sized by the data).  Signed integers sort by value;
 * f32/f64 sort by IEEE-754 totalOrder (-NaN < -Inf < ... < -0 < +0 < ... <
 * +Inf < +NaN).  The full key range is valid (no reserved sentinel such as the
 * reference's MAXVAL, src/cmp.hxx:26).
 * ------------------------------------------------------------------------- */
int gms_sort_i32(int32_t* input, int32_t* output, int64_t n, int thread_blocks, void* stream);
int gms_sort_u32(uint32_t* input, uint32_t* output, int64_t n, int thread_blocks, void* stream);
int gms_sort_i64(int64_t* input, int64_t* output, int64_t n, int thread_blocks, void* stream);
int gms_sort_u64(uint64_t* input, uint64_t* output, int64_t n, int thread_blocks, void* stream);
int gms_sort_f32(float* input, float* output, int64_t n, int thread_blocks, void* stream);
int gms_sort_f64(double* input, double* output, int64_t n, int thread_blocks, void* stream);

/* ---------------------------------------------------------------------------
 * Key/value sorts: keys with an int32 payload, stable (equal keys keep their
 * input order), i.e. the order of std::stable_sort by key.
 *
 * Replaces: the packed key/value DATATYPE of the plugin surface (a 32-bit key
 * and 32-bit value cast to 64 bits for __shfl), src/cmp.hxx:59-73, sorted by
 * multimergesort, src/multimergesort.hxx:56-141.
 *
 * keys_in/vals_in are clobbered; the result is in keys_out/vals_out.
 * ------------------------------------------------------------------------- */
int gms_sort_kv_i32_i32(int32_t* keys_in, int32_t* vals_in, int32_t* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);
int gms_sort_kv_u32_i32(uint32_t* keys_in, int32_t* vals_in, uint32_t* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);
int gms_sort_kv_f32_i32(float* keys_in, int32_t* vals_in, float* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);
int gms_sort_kv_i64_i32(int64_t* keys_in, int32_t* vals_in, int64_t* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);
int gms_sort_kv_u64_i32(uint64_t* keys_in, int32_t* vals_in, uint64_t* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);
int gms_sort_kv_f64_i32(double* keys_in, int32_t* vals_in, double* keys_out, int32_t* vals_out, int64_t n,
                        int thread_blocks, void* stream);

/* ---------------------------------------------------------------------------
 * Allocation-free int32 sort.  No counterpart in the reference (its
 * multimergesort allocates its pivots array with cudaMalloc on every call,
 * src/multimergesort.hxx:62-63).
 *
 * For callers that cannot allocate device memory while they run -- a
 * latency-critical serving loop, where cudaMalloc/cudaFree can synchronize the
 * device and stall other streams, or a host framework that fixes each plugin's
 * memory at start-up and forbids allocation in its callbacks.  Same contract
 * as gms_sort_i32 (result in `output`, `input` clobbered), but every byte of
 * scratch lives in one static 4 MiB device array of the library, held by each
 * GPU that loads it until the process exits.  Limits and rules:
 *   - n <= GMS_NOALLOC_MAX_N, else GMS_ERR_TOO_LARGE; always the default
 *     tuning (fan-in 32, sample block 32), whatever gms_set_tune says;
 *   - the first call on a device (with that device current) looks up the
 *     array's device address; make it before any stream capture;
 *   - all calls share the array: calls whose GPU work overlaps race, so order
 *     them (one stream, or explicit events).
 * It calls no cudaMalloc, cudaFree or other allocating routine.
 * ------------------------------------------------------------------------- */
#define GMS_NOALLOC_MAX_N ((int64_t)1 << 22)
int gms_sort_i32_noalloc(int32_t* input, int32_t* output, int64_t n, void* stream);
/* Waits for `stream`, then reads and clears the device status word of the
 * allocation-free sort's static array (the bits of gms_device_status, which
 * does not see this path: it reads the per-stream scratch instead).  Copies
 * into a host variable; allocates nothing.  gms_release_workspaces makes the
 * next call look the array's address up again (needed after a device reset). */
int gms_noalloc_status(void* stream, int* status_out);

/* ---------------------------------------------------------------------------
 * End-to-end sorts from host memory: copy n keys from `host_in` to the device,
 * sort, copy the result to `host_out` (may equal host_in), and wait for the
 * stream.  Device buffers come from the library's per-stream cache (allocated
 * on first use, reused afterwards).  Pinned host memory gives full copy speed.
 * gms_sort_host_i32 copies the input in up to 16 pieces (small first and
 * last) on a second stream and sorts each piece as far as it can on its own
 * (base case and early merge rounds), on two further streams in turn, as soon
 * as it lands; the last merge round runs in 8 parts, and the output prefix
 * each part makes final is copied back while the next part merges.
 *
 * Replaces: the reference's driver sequence cudaMemcpy H2D -> multimergesort
 * -> cudaMemcpy D2H, src/testMM.cu:167-195.
 * ------------------------------------------------------------------------- */
int gms_sort_host_i32(const int32_t* host_in, int32_t* host_out, int64_t n, void* stream);
/* Pipelined form (no reference counterpart): enqueues the same copy-in, sort
 * (early merge rounds on the whole array: the pipeline already overlaps the
 * copies with the neighbouring sorts) and copy-out and returns at once;
 * `host_out` holds the result, and `host_in` may be reused, after
 * gms_host_sync(stream).  Calls on one stream take three sets of device
 * buffers in turn, so the input copy of one call, the sort of the call before
 * it and the output copy of the call before that proceed together; a call's
 * input copy waits (on the device, not the host) for the output copy of the
 * call three back.  The input copy is not ordered after earlier work on
 * `stream`, so `host_in` must be ready when the call is made.  Use pinned
 * host memory (pageable memory makes the copies synchronous). */
int gms_sort_host_i32_async(const int32_t* host_in, int32_t* host_out, int64_t n, void* stream);
int gms_host_sync(void* stream);
int gms_sort_host_kv_u64_i32(const uint64_t* keys_in, const int32_t* vals_in, uint64_t* keys_out,
                             int32_t* vals_out, int64_t n, void* stream);

/* ---------------------------------------------------------------------------
 * Base case alone: every `tile`-key tile of `data` sorted in place, plus the
 * short tail tile (1 <= tile <= gms_max_tile()).
 *
 * Replaces: squareSort<T,f><<<N/M, ...>>>(data, N)
 *   src/basecase/squareSort.hxx:62-131 (tile M = 1024, tail 69-87).
 * ------------------------------------------------------------------------- */
int gms_tile_sort_i32(int32_t* data, int64_t n, int64_t tile, void* stream);
int gms_tile_sort_u64(uint64_t* data, int64_t n, int64_t tile, void* stream);
/* Largest tile the base case sorts in one CTA (keys of 4 bytes). */
int64_t gms_max_tile(void);

/* ---------------------------------------------------------------------------
 * One merge round: every group of `k` consecutive sorted runs of `run_len`
 * keys (the last run and the last group may be short) merged into one sorted
 * run of up to k*run_len keys, stably (earlier run first on ties).
 * 2 <= k <= 32.  `input` is not modified.
 *
 * Replaces: one iteration of the round loop, src/multimergesort.hxx:87-135:
 *   findPartitions + multimergeLevel<T,f>(data, output, pivots, size, tasks)
 *   src/multimergesort.hxx:155-209, src/io-merge-gen.hxx:306-355.
 * ------------------------------------------------------------------------- */
int gms_merge_level_i32(const int32_t* input, int32_t* output, int64_t n, int64_t run_len, int k, void* stream);
int gms_merge_level_u64(const uint64_t* input, uint64_t* output, int64_t n, int64_t run_len, int k, void* stream);

/* ---------------------------------------------------------------------------
 * Splitter: for one task of `k` sorted runs of `size` keys (`task_size` keys in
 * all; the last run may be short) and each target output rank r in `ranks`
 * (device, `nranks` entries), the number of keys each run contributes to the
 * first r outputs of the stable merge: out[q*k + j] (device, int64).
 * Ranks are clamped to [0, task_size].
 *
 * Replaces: findPartitions<T,f>(data, pivots, size, tasks, edgeCaseTaskSize)
 *   src/warp-partition.hxx:488-532 (single_pivot_partition 179-366), whose
 *   targets are the equal shares mergerIdInTask*taskSize/mergersPerTask
 *   (warp-partition.hxx:234); callers pass those ranks explicitly.
 * ------------------------------------------------------------------------- */
int gms_find_partitions_i32(const int32_t* task, int64_t size, int k, int64_t task_size, const int64_t* ranks,
                            int64_t nranks, int64_t* out, void* stream);

/* ---------------------------------------------------------------------------
 * Batched (segmented) sorts: `n` keys forming `nseg` independent arrays;
 * array s is [offsets[s], offsets[s+1]) with offsets[0] = 0 and
 * offsets[nseg] = n (device int64, nseg+1 entries; empty arrays allowed).
 * Every array is sorted into the same range of `output` (payload sorts:
 * stably, with the payload); the inputs are not modified.
 *
 * Each array gets its own base-case tiles and merge rounds -- no group of a
 * round crosses an array's end -- and every round is one launch sequence
 * over all the arrays that still need it: an array of at most one base tile
 * (gms_base_tile) is sorted in a single pass, one of up to 32 tiles in one
 * merge round, larger ones in rounds bounded to the array.  The call reads
 * the offsets back to plan the batch (it waits for `stream` to reach them),
 * then enqueues the sort asynchronously.  Offsets that do not rise from 0 to
 * n are GMS_ERR_INVALID; an array longer than 2^31 - 1 keys is
 * GMS_ERR_TOO_LARGE (sort it with a plain call).  Scratch: about n keys
 * (+ payload) beyond a plain sort's, from the per-stream cache.
 *
 * No counterpart in the reference: GPU-MMS sorts one array per
 * multimergesort call (src/multimergesort.hxx:56-141), each running the
 * round loop of multimergesort.hxx:87-135 on its own.
 * ------------------------------------------------------------------------- */
int gms_segmented_sort_i32(const int32_t* input, int32_t* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_u32(const uint32_t* input, uint32_t* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_f32(const float* input, float* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_i64(const int64_t* input, int64_t* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_u64(const uint64_t* input, uint64_t* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_f64(const double* input, double* output, int64_t n, const int64_t* offsets, int64_t nseg,
                           void* stream);
int gms_segmented_sort_kv_i32_i32(const int32_t* keys_in, const int32_t* vals_in, int32_t* keys_out, int32_t* vals_out,
                                  int64_t n, const int64_t* offsets, int64_t nseg, void* stream);
int gms_segmented_sort_kv_u32_i32(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out,
                                  int32_t* vals_out, int64_t n, const int64_t* offsets, int64_t nseg, void* stream);
int gms_segmented_sort_kv_f32_i32(const float* keys_in, const int32_t* vals_in, float* keys_out, int32_t* vals_out,
                                  int64_t n, const int64_t* offsets, int64_t nseg, void* stream);
int gms_segmented_sort_kv_i64_i32(const int64_t* keys_in, const int32_t* vals_in, int64_t* keys_out, int32_t* vals_out,
                                  int64_t n, const int64_t* offsets, int64_t nseg, void* stream);
int gms_segmented_sort_kv_u64_i32(const uint64_t* keys_in, const int32_t* vals_in, uint64_t* keys_out,
                                  int32_t* vals_out, int64_t n, const int64_t* offsets, int64_t nseg, void* stream);
int gms_segmented_sort_kv_f64_i32(const double* keys_in, const int32_t* vals_in, double* keys_out, int32_t* vals_out,
                                  int64_t n, const int64_t* offsets, int64_t nseg, void* stream);

/* ---------------------------------------------------------------------------
 * CUDA graphs: capture the whole launch sequence of one sort (fixed pointers
 * and sizes) and replay it with a single cudaGraphLaunch.  Creation runs the
 * sort once outside capture (setting kernel attributes and sizing scratch;
 * `input` is clobbered as by any sort), then captures it on `stream` (which
 * must not be the legacy default stream).  Replaying re-sorts whatever
 * `input` then holds into `output`.  A batched graph plans the batch from
 * the offsets at creation (the offsets must not change afterwards) and owns
 * its scratch, which gms_graph_destroy frees.
 * No counterpart in the reference (it launches every kernel from the host
 * loop, src/multimergesort.hxx:87-135).
 * ------------------------------------------------------------------------- */
typedef struct gms_graph gms_graph;
int gms_graph_create_sort_i32(int32_t* input, int32_t* output, int64_t n, void* stream, gms_graph** graph);
int gms_graph_create_segmented_i32(int32_t* input, int32_t* output, int64_t n, const int64_t* offsets,
                                   int64_t nseg, void* stream, gms_graph** graph);
int gms_graph_launch(gms_graph* graph, void* stream);
int gms_graph_destroy(gms_graph* graph);

/* ---------------------------------------------------------------------------
 * Sort server: continuous batching of device-resident requests.
 * No counterpart in the reference (a synchronous one-call-per-array library,
 * src/multimergesort.hxx:56-141).
 *
 * gms_server_create starts a dispatcher and a completion thread on the current
 * device with `nstreams` streams.  Requests (gms_server_submit) are device
 * buffers: kind 0 = int32 keys, kind 1 = uint64 keys + int32 payload (stable);
 * inputs are never modified; results go to the caller's output buffers.
 * Requests of one kind of at most `batch_max_keys` keys that wait together
 * are sorted as ONE batched sort (planned on the host, its plan uploaded from
 * pinned memory); larger requests run one per work item.  A work item starts only when its staging memory (stream-ordered
 * cudaMallocAsync) fits what is left of `memory_budget`; items run on the
 * stream pool concurrently while new requests keep arriving.  Each stream's
 * sort scratch is reserved at creation for `max_request_keys` keys (outside
 * the budget), so nothing allocates with cudaMalloc while serving.
 * gms_server_wait blocks until one request is done and gives its latency
 * (submit to completion); gms_server_stats reports p50/p99 latency and keys/s.
 * ------------------------------------------------------------------------- */
typedef struct gms_server gms_server;
int gms_server_create(size_t memory_budget, int nstreams, int64_t batch_max_keys, int64_t max_request_keys,
                      gms_server** server);
int gms_server_submit(gms_server* server, int kind, const void* keys_in, const int32_t* vals_in, void* keys_out,
                      int32_t* vals_out, int64_t n, uint64_t* request_id);
int gms_server_wait(gms_server* server, uint64_t request_id, double* latency_ms);
int gms_server_drain(gms_server* server);
int gms_server_stats(gms_server* server, int64_t* completed, double* p50_ms, double* p99_ms, double* keys_per_s);
int gms_server_destroy(gms_server* server);

/* ---------------------------------------------------------------------------
 * Scratch management.  Sorts draw device scratch from a per-(device, stream)
 * cache that grows on demand; reserve it ahead of CUDA-graph capture with
 * gms_reserve().  gms_release_workspaces() frees every cached buffer (call it
 * only when no sort is in flight).
 * ------------------------------------------------------------------------- */
/* dtype codes: 0=i32 1=u32 2=f32 3=i64 4=u64 5=f64; kv: 1 = with int32 payload.
 * gms_reserve also accepts GMS_RESERVE_SEGMENTED_I32 (batched 32-bit sorts of
 * up to n keys in all: the scratch array of n keys and a plain sort's scratch;
 * batches of many short arrays can need somewhat more). */
#define GMS_RESERVE_SEGMENTED_I32 6
size_t gms_workspace_bytes(int dtype, int kv, int64_t n);
int gms_reserve(int dtype, int kv, int64_t n, void* stream);
void gms_release_workspaces(void);

/* Programmatic dependent launch (process-wide, on by default): the sort
 * kernels go out with programmatic stream serialization, so each kernel's
 * launch is set up while the previous one runs and its CTAs start as that
 * kernel's CTAs exit, waiting on the device for its results (shorter gaps
 * between the kernels: int32 2^20 keys 0.095 instead of 0.116 ms, 2^24 0.457
 * instead of 0.490 ms on GB300).  gms_set_pdl(0) launches them in plain stream
 * order.  No counterpart in the reference, whose kernels launch with <<<>>>. */
int gms_set_pdl(int on);
int gms_get_pdl(void);

/* Explicit workspace (for serving layers that own their memory): one sort of
 * `dtype`/`kv` (codes above; vals NULL when kv = 0) that uses `workspace`, a
 * 256-byte-aligned device buffer of at least gms_workspace_bytes(dtype, kv, n)
 * bytes (query it after any gms_set_tune / gms_autotune that could change the
 * tuning of this size), instead of the per-stream cache: the call allocates
 * nothing.  Its first 256 bytes are the status word of this workspace, cleared
 * by the call; gms_workspace_status reads (and clears) it like
 * gms_device_status.  A too-small or misaligned workspace is GMS_ERR_INVALID.
 * Calls sharing one workspace must be ordered (one stream).
 * Replaces the reference's per-call cudaMalloc/cudaFree of its pivot array
 * (src/multimergesort.hxx:62,138). */
int gms_sort_ws(int dtype, int kv, void* keys_in, int32_t* vals_in, void* keys_out, int32_t* vals_out, int64_t n,
                void* workspace, size_t workspace_bytes, void* stream);
int gms_workspace_status(void* workspace, void* stream, int* status_out);

/* Waits for `stream`, then reads and clears the device status word of the
 * stream's scratch: 0 = no kernel reported a problem;
 *   bit 0 (1) = a tile exceeded the shared-memory capacity and was skipped;
 *   bit 1 (2) = a tile boundary lay outside its run;
 *   bit 2 (4) = a bulk copy into shared memory did not complete within the
 *               spin limit of its wait, and its tile was skipped (any sort,
 *               merge round or tile sort).
 * Any bit set means the result is wrong (never expected).  (A batched sort's
 * offsets are checked on the host before anything is launched: bad offsets
 * are the call's GMS_ERR_INVALID.)  Sorts with a caller-provided workspace report in that
 * workspace (gms_workspace_status), the allocation-free sort in its static
 * array (gms_noalloc_status).
 * No reference counterpart (the reference reports nothing from its kernels). */
int gms_device_status(void* stream, int* status_out);

/* ---------------------------------------------------------------------------
 * Instrumentation (no reference counterpart: the reference times the whole
 * call with cudaEvents in its driver, src/testMM.cu:170-186).
 * Kernel classes: 0 base-case tile sort, 1 data merge round, 2 sample merge,
 * 3 splitter, 4 sample gather, 5 co-rank; and two classes that are copies,
 * not kernels, of the host-to-host sorts: 6 input (host to device), 7 output
 * (device to host).
 * ------------------------------------------------------------------------- */
/* Total kernels this library has launched in the process (copies excluded). */
long long gms_launch_count(void);
/* While on, every launch (and every copy of a host-to-host sort) is
 * bracketed by CUDA events on its own stream. */
int gms_timing_enable(int on);
/* Waits for the recorded events and returns, per class (up to nclasses
 * entries), the accumulated milliseconds and timed launches; the recorded
 * launches are then consumed. */
int gms_timing_collect(double* ms, long long* launches, int nclasses);
/* The recorded launches not yet collected, in launch order: class, start and
 * end in milliseconds from the earliest start (one device clock across
 * streams).  Fills up to max_entries and returns how many were recorded, or
 * a negative status.  Call before gms_timing_collect. */
int gms_timing_trace(int* classes, double* start_ms, double* end_ms, int max_entries);
int gms_timing_reset(void);

/* ---------------------------------------------------------------------------
 * Tuning, process-wide, applied to calls that start afterwards.
 * Replaces the reference's compile-time constants K (fan-in) and PIPELINE /
 * BLOCKS (src/params.h:18-20), which its sweep scripts tried to override
 * (scripts/findK.sh, scripts/blocksThreads.sh).
 *   k          fan-in of a merge round, 2..32 (default 32)
 *   sample_b   block size of the forecast sample that cuts tiles (default 32;
 *              8 <= sample_b and 4080/sample_b > k, 4080 keys being the
 *              smallest merge-tile capacity of the prebuilt engines).  A sort whose sample
 *              recursion would get too deep for the tuning returns
 *              GMS_ERR_INVALID.
 *   bulk_copy  how the merge kernel stages a tile's segments in shared
 *              memory: 1 one cp.async.bulk per segment issued by one warp
 *              (default); 3 the same with persistent CTAs that stage the
 *              next tile while storing the current one; 2 16-byte cp.async
 *              issued by every warp; 0 a merge kernel with plain loads
 * Out-of-range values (k outside [2, 32], sample_b below 8 or too large for
 * k, bulk_copy outside [0, 3]) return GMS_ERR_INVALID and change nothing.
 * A tuning set here applies to every dtype and size until gms_clear_tune,
 * which returns to the autotuned table below and, for classes it does not
 * hold, the built-in defaults (k 32, sample_b 32, bulk_copy 1; bulk_copy 3
 * for sorts with a payload).
 * ------------------------------------------------------------------------- */
int gms_set_tune(int k, int sample_b, int bulk_copy);
int gms_get_tune(int* k, int* sample_b, int* bulk_copy);
int gms_clear_tune(void);
/* The same with two strategy switches, the counterparts of the reference's
 * compile-time alternatives:
 *   split  tile boundaries (PIVOT_MOVES, src/params.h:21; the partition
 *          strategies of src/warp-partition.hxx:179-470):
 *            0  each run's co-rank bracketed to one block by the run's block
 *               sample, then searched inside it (default);
 *            1  a binary search over the whole run, as findPartitions does;
 *   base   base case of keys-only sorts (the base-case variants of
 *          src/basecase/squareSort.hxx:62-131, sortRowMajor.hxx:341-392):
 *            0  register network per lane + warp-shuffle merges + shared-memory
 *               levels, 8192-key tiles for 32-bit keys (default);
 *            1  register network per thread + shared-memory merge levels,
 *               8704-key tiles (the base case of the payload engines).
 * gms_set_tune sets both to 0.  The autotuner tries split 1 and then base 1
 * on its best tuning. */
int gms_set_tune_ex(int k, int sample_b, int bulk_copy, int split, int base);
int gms_get_tune_ex(int* k, int* sample_b, int* bulk_copy, int* split, int* base);

/* ---------------------------------------------------------------------------
 * Autotuner.  No reference counterpart beyond the sweep scripts named above:
 * the reference fixes K/PIPELINE/BLOCKS at compile time (src/params.h:18-20).
 *
 * gms_autotune times every candidate tuning (k in {8,16,32}, sample_b in
 * {16,32,64}, the three staging modes) on a sort of n synthetic keys of `dtype`
 * (0 i32, 1 u32, 2 f32, 3 i64, 4 u64, 5 f64; kv=1: with int32 values) on
 * `stream`, checks that all tunings give the same bits, and records the
 * fastest (median of repeats) for the size class floor(log2 n).  Later sorts
 * of that dtype, payload and size class use it unless gms_set_tune is in
 * force.  Synchronous; allocates its own buffers (about 3 arrays of n keys and
 * values) and frees them before returning.
 * gms_tune_for reports the tuning a sort of (dtype, kv, n) would use.
 * gms_autotune_table writes the table as JSON into buf (needed = bytes with
 * the terminating NUL; buf may be NULL to query the size).
 * gms_autotune_save / _load write / read the table as a JSON file recorded
 * with the GPU's name; a file recorded on another GPU model is refused
 * (GMS_ERR_INVALID).  If the environment variable GMS_TUNE_CACHE names such a
 * file, it is loaded before the first sort of the process.
 * ------------------------------------------------------------------------- */
int gms_autotune(int dtype, int kv, int64_t n, void* stream, int* out_k, int* out_sample_b, int* out_bulk_copy,
                 double* out_ms);
int gms_tune_for(int dtype, int kv, int64_t n, int* k, int* sample_b, int* bulk_copy);
int gms_autotune_table(char* buf, size_t cap, size_t* needed);
int gms_autotune_clear(void);
int gms_autotune_save(const char* path);
int gms_autotune_load(const char* path);

/* Number of merge rounds (after the base case) a sort of n keys of the given
 * dtype performs, and the base tile (keys) it uses. */
int gms_rounds(int dtype, int kv, int64_t n);
int64_t gms_base_tile(int dtype, int kv);

#ifdef __cplusplus
}
#endif

#endif /* GMS_H_ */
