"""The allocation-free sort (gms_sort_i32_noalloc), called through the C ABI.

It exists for callers that must not allocate device memory while they run
(a serving loop where cudaMalloc/cudaFree would synchronize the device and
stall other streams, or a host that fixes each plugin's memory at start-up):
the sort keeps its scratch in one static device array of the library.  Its
output must equal the oracle's std::sort and the ordinary gms_sort_i32 output
bit for bit, call after call, since every call reuses the same array; and the
calls must leave the device's free memory unchanged.  This file is collected
last so that a run stopping at the first failure has run every other test
first.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sort(lib, fn, a):
    tin = torch.from_numpy(a.copy()).cuda()
    tout = torch.empty_like(tin)
    rc = getattr(lib, fn)(tin.data_ptr(), tout.data_ptr(), a.size, *([0] if fn == "gms_sort_i32" else []), _stream())
    assert rc == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    return tout.cpu().numpy()


def _noalloc_status(lib):
    st = ctypes.c_int(-1)
    assert lib.gms_noalloc_status(_stream(), ctypes.byref(st)) == 0, lib.gms_last_error()
    return st.value


def test_no_alloc_sort_matches_oracle_and_plain_sort_twice(gms, oracle):
    lib = gms.load()
    max_n = 1 << 22
    # two calls in a row on the shared scratch, different sizes and inputs
    for n, dist, seed in [(max_n, 6, 11), (1_000_003, 4, 12)]:
        a = oracle.gen_i32(n, dist, seed)
        want = oracle.sort(a)
        got = _sort(lib, "gms_sort_i32_noalloc", a)
        assert _noalloc_status(lib) == 0
        assert np.array_equal(got, want), f"n={n}: differs from the oracle"
        assert np.array_equal(got, _sort(lib, "gms_sort_i32", a)), f"n={n}: differs from gms_sort_i32"
    # and once more on the first input: results do not depend on leftovers
    a = oracle.gen_i32(max_n, 6, 11)
    assert np.array_equal(_sort(lib, "gms_sort_i32_noalloc", a), oracle.sort(a))


def test_no_alloc_leaves_free_memory_unchanged(gms, oracle):
    lib = gms.load()
    n = 1 << 22
    a = oracle.gen_i32(n, 0, 21)
    src = torch.from_numpy(a).cuda()
    tin = torch.empty_like(src)
    tout = torch.empty_like(src)
    sp = _stream()
    # drop the library's scratch cache; the first call looks up the static
    # array's address (and loads the kernels), so it runs before the measurement
    lib.gms_release_workspaces()
    tin.copy_(src)
    assert lib.gms_sort_i32_noalloc(tin.data_ptr(), tout.data_ptr(), n, sp) == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        tin.copy_(src)
        assert lib.gms_sort_i32_noalloc(tin.data_ptr(), tout.data_ptr(), n, sp) == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert _noalloc_status(lib) == 0
    assert np.array_equal(tout.cpu().numpy(), oracle.sort(a))


def test_no_alloc_rejects_beyond_limit(gms):
    lib = gms.load()
    t = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = lib.gms_sort_i32_noalloc(t.data_ptr(), t.data_ptr(), (1 << 22) + 1, _stream())
    assert rc == 4  # GMS_ERR_TOO_LARGE
    assert b"GMS_NOALLOC_MAX_N" in lib.gms_last_error()
