"""The allocation-free sort (gms_sort_i32_noalloc), called through the C ABI.

It exists for callers that must not allocate device memory while they run
(a serving loop where cudaMalloc/cudaFree would synchronize the device and
stall other streams, or a host that fixes each plugin's memory at start-up):
the sort keeps its scratch in one static device array of the library.  Its
output must equal the ordinary gms_sort_i32 output bit for bit, call after
call, since every call reuses the same array.  This file is collected last
so that a run stopping at the first failure has run every other test first.
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
    rc = getattr(lib, fn)(tin.data_ptr(), tout.data_ptr(), a.size, *( [0] if fn == "gms_sort_i32" else []), _stream())
    assert rc == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    return tout.cpu().numpy()


def test_no_alloc_sort_matches_plain_sort_twice(gms, oracle):
    lib = gms.load()
    max_n = 1 << 22
    # two calls in a row on the shared scratch, different sizes and inputs
    for n, dist, seed in [(max_n, 6, 11), (1_000_003, 4, 12)]:
        a = oracle.gen_i32(n, dist, seed)
        want = _sort(lib, "gms_sort_i32", a)
        got = _sort(lib, "gms_sort_i32_noalloc", a)
        assert np.array_equal(got, want), f"n={n}"
    # and once more on the first input: results do not depend on leftovers
    a = oracle.gen_i32(max_n, 6, 11)
    assert np.array_equal(_sort(lib, "gms_sort_i32_noalloc", a), _sort(lib, "gms_sort_i32", a))


def test_no_alloc_rejects_beyond_limit(gms):
    lib = gms.load()
    t = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = lib.gms_sort_i32_noalloc(t.data_ptr(), t.data_ptr(), (1 << 22) + 1, _stream())
    assert rc == 4  # GMS_ERR_TOO_LARGE
    assert b"GMS_NOALLOC_MAX_N" in lib.gms_last_error()
