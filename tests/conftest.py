"""Shared fixtures.  `gpu`-marked tests need a CUDA device and call the CUDA
library only through its C ABI (gpu-mms_gb300/libgms.so); the oracle
(oracle/liboracle.so) gives the expected results."""
import ctypes
import importlib.util
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def load_gms_module():
    spec = importlib.util.spec_from_file_location("gms", os.path.join(ROOT, "gpu-mms_gb300", "gms.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_oracle = None


def load_oracle():
    global _oracle
    if _oracle is not None:
        return _oracle
    src = os.path.join(ROOT, "oracle", "oracle.cpp")
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    lib = ctypes.CDLL(ORACLE_SO)
    vp, i64, u64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int
    sigs = {
        "gmo_sort_i32": [vp, i64], "gmo_sort_u32": [vp, i64], "gmo_sort_i64": [vp, i64],
        "gmo_sort_u64": [vp, i64], "gmo_sort_f32": [vp, i64], "gmo_sort_f64": [vp, i64],
        "gmo_sort_kv_u32_i32": [vp, vp, i64], "gmo_sort_kv_i32_i32": [vp, vp, i64],
        "gmo_sort_kv_u64_i32": [vp, vp, i64], "gmo_sort_kv_i64_i32": [vp, vp, i64],
        "gmo_sort_kv_f32_i32": [vp, vp, i64], "gmo_sort_kv_f64_i32": [vp, vp, i64],
        "gmo_segmented_sort_i32": [vp, vp, i64], "gmo_segmented_sort_u64": [vp, vp, i64],
        "gmo_segmented_sort_kv_u64_i32": [vp, vp, vp, i64],
        "gmo_tile_sort_i32": [vp, i64, i64], "gmo_tile_sort_u64": [vp, i64, i64],
        "gmo_merge_level_i32": [vp, vp, i64, i64, i32], "gmo_merge_level_u64": [vp, vp, i64, i64, i32],
        "gmo_find_partitions_i32": [vp, i64, i32, i64, vp, i64, vp],
        "gmo_ref_random_list": [vp, i64, ctypes.c_uint], "gmo_selection_sort_i32": [vp, i64],
        "gmo_gen_i32": [vp, i64, i32, u64], "gmo_gen_u64": [vp, i64, u64], "gmo_gen_f32": [vp, i64, u64],
        "gmo_gen_seg_lengths": [vp, i64, i64, i64, u64],
        "gmo_first_diff": [vp, vp, i64, i32],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = None
    lib.gmo_gen_seg_lengths.restype = i64
    lib.gmo_first_diff.restype = i64
    lib.gmo_par_sort_i32.argtypes = [vp, i64, i32]
    lib.gmo_par_sort_i32.restype = ctypes.c_double
    lib.gmo_max_threads.restype = i32
    _oracle = lib
    return lib


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Oracle:
    """numpy-facing wrapper of oracle/liboracle.so."""

    def __init__(self):
        self.lib = load_oracle()

    def sort(self, a):
        a = np.ascontiguousarray(a).copy()
        fn = {np.dtype(np.int32): "gmo_sort_i32", np.dtype(np.uint32): "gmo_sort_u32",
              np.dtype(np.int64): "gmo_sort_i64", np.dtype(np.uint64): "gmo_sort_u64",
              np.dtype(np.float32): "gmo_sort_f32", np.dtype(np.float64): "gmo_sort_f64"}[a.dtype]
        getattr(self.lib, fn)(ptr(a), a.size)
        return a

    def sort_kv(self, k, v):
        k = np.ascontiguousarray(k).copy()
        v = np.ascontiguousarray(v, dtype=np.int32).copy()
        fn = {np.dtype(np.int32): "gmo_sort_kv_i32_i32", np.dtype(np.uint32): "gmo_sort_kv_u32_i32",
              np.dtype(np.int64): "gmo_sort_kv_i64_i32", np.dtype(np.uint64): "gmo_sort_kv_u64_i32",
              np.dtype(np.float32): "gmo_sort_kv_f32_i32", np.dtype(np.float64): "gmo_sort_kv_f64_i32"}[k.dtype]
        getattr(self.lib, fn)(ptr(k), ptr(v), k.size)
        return k, v

    def segmented_sort(self, a, off):
        """Every [off[s], off[s+1]) sorted on its own (int32 or uint64 keys)."""
        a = np.ascontiguousarray(a).copy()
        off = np.ascontiguousarray(off, dtype=np.int64)
        fn = {np.dtype(np.int32): "gmo_segmented_sort_i32", np.dtype(np.uint64): "gmo_segmented_sort_u64"}[a.dtype]
        getattr(self.lib, fn)(ptr(a), ptr(off), len(off) - 1)
        return a

    def segmented_sort_kv_u64(self, k, v, off):
        """Every [off[s], off[s+1]) sorted stably by its uint64 keys, int32 payload along."""
        k = np.ascontiguousarray(k, dtype=np.uint64).copy()
        v = np.ascontiguousarray(v, dtype=np.int32).copy()
        off = np.ascontiguousarray(off, dtype=np.int64)
        self.lib.gmo_segmented_sort_kv_u64_i32(ptr(k), ptr(v), ptr(off), len(off) - 1)
        return k, v

    def tile_sort(self, a, tile):
        a = np.ascontiguousarray(a).copy()
        fn = self.lib.gmo_tile_sort_i32 if a.dtype == np.int32 else self.lib.gmo_tile_sort_u64
        fn(ptr(a), a.size, tile)
        return a

    def merge_level(self, a, run_len, k):
        a = np.ascontiguousarray(a)
        out = np.empty_like(a)
        fn = self.lib.gmo_merge_level_i32 if a.dtype == np.int32 else self.lib.gmo_merge_level_u64
        fn(ptr(a), ptr(out), a.size, run_len, k)
        return out

    def find_partitions(self, task, size, k, ranks):
        task = np.ascontiguousarray(task, dtype=np.int32)
        ranks = np.ascontiguousarray(ranks, dtype=np.int64)
        out = np.zeros((ranks.size, k), dtype=np.int64)
        self.lib.gmo_find_partitions_i32(ptr(task), size, k, task.size, ptr(ranks), ranks.size, ptr(out))
        return out

    def gen_i32(self, n, dist, seed):
        a = np.empty(n, dtype=np.int32)
        self.lib.gmo_gen_i32(ptr(a), n, dist, seed)
        return a

    def gen_u64(self, n, seed):
        a = np.empty(n, dtype=np.uint64)
        self.lib.gmo_gen_u64(ptr(a), n, seed)
        return a

    def gen_f32(self, n, seed):
        a = np.empty(n, dtype=np.float32)
        self.lib.gmo_gen_f32(ptr(a), n, seed)
        return a

    def ref_random_list(self, n, seed):
        a = np.empty(max(n, 1), dtype=np.int32)
        self.lib.gmo_ref_random_list(ptr(a), n, seed)
        return a[:n]

    def selection_sort(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32).copy()
        self.lib.gmo_selection_sort_i32(ptr(a), a.size)
        return a


@pytest.fixture(scope="session")
def oracle():
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_random_list.npz"))


@pytest.fixture(scope="session")
def gms():
    """The C-ABI binding with libgms.so built and loaded (GPU tests only)."""
    mod = load_gms_module()
    mod.build()
    mod.load()
    return mod
