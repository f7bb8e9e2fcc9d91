"""Python binding of the GB300 multiway mergesort C ABI (include/gms.h).

Builds libgms.so from csrc/ with nvcc for sm_103a and exposes the C entry
points through ctypes.  PyTorch supplies device memory and the current CUDA
stream; no compute happens in Python.  There is no CPU fallback: if the shared
library is missing or fails to load, every call raises.

Reference interface mirrored: multimergesort<T,cmp>(input, output, host_array,
threadBlocks, N) (GPU-MMS src/multimergesort.hxx:56-141, README.md:16-25),
squareSort (src/basecase/squareSort.hxx:62-131), one merge round
(src/multimergesort.hxx:87-135, 155-209) and findPartitions
(src/warp-partition.hxx:488-532).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgms.so")
CLI = os.path.join(HERE, "testmm")
THRUST = os.path.join(HERE, "thrust_baseline")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC"]
UNITS = ["gms_capi_misc.cu", "gms_capi_k32.cu", "gms_capi_k64.cu", "gms_capi_kv.cu", "gms_capi_noalloc.cu",
         "gms_capi_seg.cu", "gms_capi_tune.cu", "gms_server.cu"]

GMS_OK = 0
DTYPES = {"int32": 0, "uint32": 1, "float32": 2, "int64": 3, "uint64": 4, "float64": 5}


class GmsError(RuntimeError):
    """A C-ABI call returned a non-zero gms_status."""

    def __init__(self, status, where, message):
        super().__init__(f"{where}: status {status}: {message}")
        self.status = status


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources():
    out = []
    for d in (CSRC, INCLUDE, os.path.join(HERE, "cli")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".hxx")):
                out.append(os.path.join(d, f))
    return out


def _source_hash():
    """SHA-256 over every source file (path and bytes), the compiler flags and
    the unit list: the build's identity, independent of file times."""
    h = hashlib.sha256()
    for p in sorted(_sources()):
        h.update(os.path.relpath(p, ROOT).encode())
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(repr((NVCC_FLAGS, UNITS)).encode())
    return h.hexdigest()


def build(force=False, jobs=None, verbose=False):
    """Compile csrc/*.cu for sm_103a into libgms.so (in-tree).  Skipped only
    when libgms.so and the command-line programs exist and were built from
    sources with the same hash (recorded in _build/sources.sha256)."""
    os.makedirs(BUILD, exist_ok=True)
    digest = _source_hash()
    stamp = os.path.join(BUILD, "sources.sha256")
    built = open(stamp).read().strip() if os.path.exists(stamp) else ""
    if not force and built == digest and all(os.path.exists(p) for p in (LIB, CLI, THRUST)):
        return LIB
    if os.path.exists(stamp):
        os.unlink(stamp)
    nvcc = _nvcc()

    def compile_one(unit):
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)
        return obj

    def compile_cli():
        # testmm: the reference-compatible command-line driver (header-only path)
        cmd = [nvcc] + ARCH + ["-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", INCLUDE,
                               os.path.join(HERE, "cli", "testmm.cu"), "-o", CLI + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for testmm:\n{r.stdout}\n{r.stderr}")
        os.replace(CLI + ".tmp", CLI)

    def compile_thrust():
        # thrust_baseline: GPU library baselines (CUB radix and merge sort via thrust)
        cmd = [nvcc] + ARCH + ["-O2", "-std=c++17", "--extended-lambda",
                               os.path.join(HERE, "cli", "thrust_baseline.cu"), "-o", THRUST + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for thrust_baseline:\n{r.stdout}\n{r.stderr}")
        os.replace(THRUST + ".tmp", THRUST)

    with ThreadPoolExecutor(max_workers=jobs or len(UNITS) + 2) as ex:
        cli = ex.submit(compile_cli)
        thr = ex.submit(compile_thrust)
        objs = list(ex.map(compile_one, UNITS))
        cli.result()
        thr.result()
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest + "\n")
    return LIB


# ---------------------------------------------------------------------------
# ctypes declarations: name -> (restype, argtypes)
_i32, _i64, _u64, _vp, _sz = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t
SIGNATURES = {
    "gms_version": (_i32, []),
    "gms_status_string": (ctypes.c_char_p, [_i32]),
    "gms_last_error": (ctypes.c_char_p, []),
    "gms_sort_i32": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_u32": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_i64": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_u64": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_f32": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_f64": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_i32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_u32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_f32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_i64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_u64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_kv_f64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "gms_sort_host_i32": (_i32, [_vp, _vp, _i64, _vp]),
    "gms_sort_host_i32_async": (_i32, [_vp, _vp, _i64, _vp]),
    "gms_host_sync": (_i32, [_vp]),
    "gms_sort_i32_noalloc": (_i32, [_vp, _vp, _i64, _vp]),
    "gms_noalloc_status": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "gms_sort_host_kv_u64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp]),
    "gms_segmented_sort_i32": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_u32": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_f32": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_i64": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_u64": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_f64": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_i32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_u32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_f32_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_i64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_u64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_segmented_sort_kv_f64_i32": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "gms_graph_create_sort_i32": (_i32, [_vp, _vp, _i64, _vp, ctypes.POINTER(_vp)]),
    "gms_graph_create_segmented_i32": (_i32, [_vp, _vp, _i64, _vp, _i64, _vp, ctypes.POINTER(_vp)]),
    "gms_graph_launch": (_i32, [_vp, _vp]),
    "gms_set_pdl": (_i32, [_i32]),
    "gms_get_pdl": (_i32, []),
    "gms_server_create": (_i32, [_sz, _i32, _i64, _i64, ctypes.POINTER(_vp)]),
    "gms_server_submit": (_i32, [_vp, _i32, _vp, _vp, _vp, _vp, _i64, ctypes.POINTER(ctypes.c_uint64)]),
    "gms_server_wait": (_i32, [_vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]),
    "gms_server_drain": (_i32, [_vp]),
    "gms_server_stats": (_i32, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gms_server_destroy": (_i32, [_vp]),
    "gms_graph_destroy": (_i32, [_vp]),
    "gms_tile_sort_i32": (_i32, [_vp, _i64, _i64, _vp]),
    "gms_tile_sort_u64": (_i32, [_vp, _i64, _i64, _vp]),
    "gms_max_tile": (_i64, []),
    "gms_merge_level_i32": (_i32, [_vp, _vp, _i64, _i64, _i32, _vp]),
    "gms_merge_level_u64": (_i32, [_vp, _vp, _i64, _i64, _i32, _vp]),
    "gms_find_partitions_i32": (_i32, [_vp, _i64, _i32, _i64, _vp, _i64, _vp, _vp]),
    "gms_workspace_bytes": (_sz, [_i32, _i32, _i64]),
    "gms_reserve": (_i32, [_i32, _i32, _i64, _vp]),
    "gms_device_status": (_i32, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "gms_release_workspaces": (None, []),
    "gms_sort_ws": (_i32, [_i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _sz, _vp]),
    "gms_workspace_status": (_i32, [_vp, _vp, ctypes.POINTER(ctypes.c_int)]),
    "gms_launch_count": (ctypes.c_longlong, []),
    "gms_set_tune": (_i32, [_i32, _i32, _i32]),
    "gms_get_tune": (_i32, [ctypes.POINTER(ctypes.c_int)] * 3),
    "gms_set_tune_ex": (_i32, [_i32, _i32, _i32, _i32, _i32]),
    "gms_get_tune_ex": (_i32, [ctypes.POINTER(ctypes.c_int)] * 5),
    "gms_clear_tune": (_i32, []),
    "gms_autotune": (_i32, [_i32, _i32, _i64, _vp] + [ctypes.POINTER(ctypes.c_int)] * 3
                     + [ctypes.POINTER(ctypes.c_double)]),
    "gms_tune_for": (_i32, [_i32, _i32, _i64] + [ctypes.POINTER(ctypes.c_int)] * 3),
    "gms_autotune_table": (_i32, [ctypes.c_char_p, _sz, ctypes.POINTER(ctypes.c_size_t)]),
    "gms_autotune_clear": (_i32, []),
    "gms_autotune_save": (_i32, [ctypes.c_char_p]),
    "gms_autotune_load": (_i32, [ctypes.c_char_p]),
    "gms_timing_enable": (_i32, [_i32]),
    "gms_timing_collect": (_i32, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong), _i32]),
    "gms_timing_trace": (_i32, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double), _i32]),
    "gms_timing_reset": (_i32, []),
    "gms_rounds": (_i32, [_i32, _i32, _i64]),
    "gms_base_tile": (_i64, [_i32, _i32]),
}

_lock = threading.Lock()
_lib = None


def load(path=None):
    """Load libgms.so (raises if it is missing: there is no fallback)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB
        if not os.path.exists(p):
            raise OSError(f"{p} not found: build it with gms.build() (nvcc, sm_103a)")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def _check(status, where):
    if status != GMS_OK:
        lib = load()
        raise GmsError(status, where, lib.gms_last_error().decode(errors="replace"))


# ---------------------------------------------------------------------------
# torch-facing helpers (device tensors, current stream)
def _stream_ptr(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


_SUFFIX = {"torch.int32": "i32", "torch.uint32": "u32", "torch.float32": "f32", "torch.int64": "i64",
           "torch.uint64": "u64", "torch.float64": "f64"}


def _suffix(t):
    s = _SUFFIX.get(str(t.dtype))
    if s is None:
        raise TypeError(f"unsupported key dtype {t.dtype}")
    return s


def _dev_check(*ts):
    for t in ts:
        if not t.is_cuda or not t.is_contiguous():
            raise ValueError("tensors must be contiguous CUDA tensors")


def sort_(inp, out, thread_blocks=0, stream=None):
    """multimergesort: sorts `inp` into `out` (both device, same dtype/size).
    `inp` is clobbered.  Returns `out`."""
    _dev_check(inp, out)
    if inp.numel() != out.numel() or inp.dtype != out.dtype:
        raise ValueError("input/output mismatch")
    lib = load()
    fn = getattr(lib, "gms_sort_" + _suffix(inp))
    _check(fn(inp.data_ptr(), out.data_ptr(), inp.numel(), thread_blocks, _stream_ptr(stream)), fn.__name__)
    return out


def sort(t, stream=None):
    """Returns a sorted copy of device tensor `t` (t is left intact)."""
    import torch

    inp = t.clone()
    out = torch.empty_like(t)
    return sort_(inp, out, stream=stream)


def sort_kv_(kin, vin, kout, vout, thread_blocks=0, stream=None):
    """Stable key/value sort (int32 payload); inputs clobbered."""
    _dev_check(kin, vin, kout, vout)
    if str(vin.dtype) != "torch.int32":
        raise TypeError("payload must be int32")
    lib = load()
    fn = getattr(lib, "gms_sort_kv_" + _suffix(kin) + "_i32")
    _check(fn(kin.data_ptr(), vin.data_ptr(), kout.data_ptr(), vout.data_ptr(), kin.numel(), thread_blocks,
              _stream_ptr(stream)), fn.__name__)
    return kout, vout


def sort_kv(keys, vals, stream=None):
    import torch

    ki, vi = keys.clone(), vals.clone()
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    return sort_kv_(ki, vi, ko, vo, stream=stream)


def tile_sort_(data, tile, stream=None):
    """squareSort contract: every `tile`-key tile sorted in place."""
    _dev_check(data)
    lib = load()
    fn = {"i32": lib.gms_tile_sort_i32, "u64": lib.gms_tile_sort_u64}[_suffix(data)]
    _check(fn(data.data_ptr(), data.numel(), tile, _stream_ptr(stream)), "tile_sort")
    return data


def merge_level(inp, run_len, k, stream=None):
    """One K-way merge round over runs of `run_len`; returns a new tensor."""
    import torch

    _dev_check(inp)
    out = torch.empty_like(inp)
    lib = load()
    fn = {"i32": lib.gms_merge_level_i32, "u64": lib.gms_merge_level_u64}[_suffix(inp)]
    _check(fn(inp.data_ptr(), out.data_ptr(), inp.numel(), run_len, k, _stream_ptr(stream)), "merge_level")
    return out


def find_partitions(task, size, k, ranks, stream=None):
    """findPartitions contract: per rank, the keys each of the k runs gives."""
    import torch

    _dev_check(task, ranks)
    out = torch.empty((ranks.numel(), k), dtype=torch.int64, device=task.device)
    lib = load()
    _check(lib.gms_find_partitions_i32(task.data_ptr(), size, k, task.numel(), ranks.data_ptr(), ranks.numel(),
                                       out.data_ptr(), _stream_ptr(stream)), "find_partitions")
    return out


KERNEL_CLASSES = ["base_tile_sort", "merge_round", "sample_merge", "splitter", "sample_gather", "corank",
                  "h2d_copy", "d2h_copy"]


def timing_collect():
    """Per kernel class: (milliseconds, timed launches) since the last reset."""
    lib = load()
    n = len(KERNEL_CLASSES)
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_longlong * n)()
    _check(lib.gms_timing_collect(ms, cnt, n), "timing_collect")
    return {name: (ms[i], cnt[i]) for i, name in enumerate(KERNEL_CLASSES)}


def timing_trace(max_entries=100000):
    """Recorded launches not yet collected: [(class name, start ms, end ms)],
    in launch order, times from the earliest start.  Call before
    timing_collect(), which consumes them."""
    lib = load()
    cls = (ctypes.c_int * max_entries)()
    t0 = (ctypes.c_double * max_entries)()
    t1 = (ctypes.c_double * max_entries)()
    n = lib.gms_timing_trace(cls, t0, t1, max_entries)
    if n < 0:
        _check(n, "timing_trace")
    return [(KERNEL_CLASSES[cls[i]], t0[i], t1[i]) for i in range(min(n, max_entries))]


def device_status(stream=None):
    """Waits for the stream and returns (and clears) the device status word."""
    lib = load()
    v = ctypes.c_int(0)
    _check(lib.gms_device_status(_stream_ptr(stream), ctypes.byref(v)), "device_status")
    return v.value


def sort_host_i32(host_in, host_out, stream=None):
    """End-to-end: host int32 array in, sorted host array out (waits)."""
    lib = load()
    _check(lib.gms_sort_host_i32(host_in.data_ptr(), host_out.data_ptr(), host_in.numel(), _stream_ptr(stream)),
           "sort_host_i32")
    return host_out


def autotune(dtype, n, kv=False, stream=None):
    """Times the candidate tunings for (dtype, kv, size class of n) on the
    device and records the fastest; returns {k, sample_b, bulk_copy, ms}."""
    lib = load()
    k, b, bulk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ms = ctypes.c_double()
    _check(lib.gms_autotune(DTYPES[dtype], int(bool(kv)), int(n), _stream_ptr(stream), ctypes.byref(k),
                            ctypes.byref(b), ctypes.byref(bulk), ctypes.byref(ms)), "autotune")
    return {"k": k.value, "sample_b": b.value, "bulk_copy": bulk.value, "ms": ms.value}


def tune_for(dtype, n, kv=False):
    """The tuning a sort of (dtype, kv, n) would use now."""
    lib = load()
    k, b, bulk = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib.gms_tune_for(DTYPES[dtype], int(bool(kv)), int(n), ctypes.byref(k), ctypes.byref(b),
                            ctypes.byref(bulk)), "tune_for")
    return {"k": k.value, "sample_b": b.value, "bulk_copy": bulk.value}


def autotune_table():
    """The autotuned table as a list of dicts."""
    import json
    lib = load()
    need = ctypes.c_size_t()
    _check(lib.gms_autotune_table(None, 0, ctypes.byref(need)), "autotune_table")
    buf = ctypes.create_string_buffer(need.value)
    _check(lib.gms_autotune_table(buf, need.value, ctypes.byref(need)), "autotune_table")
    return json.loads(buf.value.decode())


def autotune_save(path):
    _check(load().gms_autotune_save(os.fsencode(path)), "autotune_save")


def autotune_load(path):
    _check(load().gms_autotune_load(os.fsencode(path)), "autotune_load")
