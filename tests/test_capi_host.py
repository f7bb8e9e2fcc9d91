"""Host-side logic of the C ABI, run without a GPU: argument checks that come
before any device work, and the process-wide tuning state (gms_set_tune /
gms_get_tune / gms_clear_tune / gms_tune_for)."""
import ctypes

import pytest

from conftest import load_gms_module

GMS_OK, GMS_ERR_INVALID = 0, 1


@pytest.fixture(scope="module")
def lib():
    mod = load_gms_module()
    mod.build()
    return mod.load()


def get_tune(lib):
    k, b, m = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert lib.gms_get_tune(ctypes.byref(k), ctypes.byref(b), ctypes.byref(m)) == GMS_OK
    return k.value, b.value, m.value


def tune_for(lib, dtype, kv, n):
    k, b, m = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert lib.gms_tune_for(dtype, kv, n, ctypes.byref(k), ctypes.byref(b), ctypes.byref(m)) == GMS_OK
    return k.value, b.value, m.value


def test_tuning_state(lib):
    try:
        assert lib.gms_clear_tune() == GMS_OK
        assert get_tune(lib) == (32, 32, 1)
        # built-in defaults per class: staging mode 3 for sorts with a payload
        assert tune_for(lib, 0, 0, 1 << 28) == (32, 32, 1)
        assert tune_for(lib, 2, 1, 1 << 27) == (32, 32, 3)
        assert lib.gms_set_tune(16, 64, 2) == GMS_OK
        assert get_tune(lib) == (16, 64, 2)
        # an explicit tuning applies to every class
        assert tune_for(lib, 0, 0, 1 << 28) == (16, 64, 2)
        assert tune_for(lib, 4, 1, 1 << 20) == (16, 64, 2)
        # rejected values change nothing and say why
        for args in [(1, 32, 1), (33, 32, 1), (32, 0, 1), (32, 7, 1), (32, 128, 1), (32, 32, -1), (32, 32, 4)]:
            assert lib.gms_set_tune(*args) == GMS_ERR_INVALID, args
            assert lib.gms_last_error() != b""
            assert get_tune(lib) == (16, 64, 2)
        assert lib.gms_set_tune(32, 32, 9) == GMS_ERR_INVALID
        assert b"bulk_copy" in lib.gms_last_error()
        for mode in range(4):
            assert lib.gms_set_tune(8, 16, mode) == GMS_OK
            assert get_tune(lib) == (8, 16, mode)
    finally:
        lib.gms_clear_tune()
    assert get_tune(lib) == (32, 32, 1)


def test_builtin_fan_in_balances_the_rounds(lib):
    """Keys-only sorts take the fewest rounds a fan-in of at most 32 allows
    and the smallest power-of-two fan-in that keeps that many rounds (block
    sample 64 below a fan-in of 32); key/value sorts keep 32 / 32."""
    lib.gms_clear_tune()
    # int32: base runs of 8192 keys
    assert tune_for(lib, 0, 0, 1 << 13) == (32, 32, 1)  # one base tile: no round
    assert tune_for(lib, 0, 0, 1 << 18) == (32, 32, 1)  # 32 runs: one round of 32
    assert tune_for(lib, 0, 0, 1 << 20) == (16, 64, 1)  # 128 runs: two rounds of 16 (not 32 + 4)
    assert tune_for(lib, 0, 0, 1 << 22) == (32, 32, 1)  # 512 runs: two rounds of 32
    assert tune_for(lib, 0, 0, 1 << 24) == (16, 64, 1)  # 2048 runs: three rounds of 16 (not 32, 32, 2)
    assert tune_for(lib, 0, 0, (1 << 24) + 1) == (16, 64, 1)  # 2049 runs: 16^3 = 4096 still covers them
    assert tune_for(lib, 1, 0, 1 << 26) == (32, 32, 1)
    assert tune_for(lib, 2, 0, 1 << 28) == (32, 32, 1)
    # 64-bit keys: base runs of 4096 keys, persistent staging
    assert tune_for(lib, 4, 0, 1 << 18) == (8, 64, 3)   # 64 runs: two rounds of 8
    assert tune_for(lib, 3, 0, 1 << 24) == (16, 64, 3)
    assert tune_for(lib, 5, 0, 1 << 22) == (32, 32, 3)
    # payload sorts: base runs of 4352 keys, block sample 64 only below fan-in 16
    assert tune_for(lib, 2, 1, 1 << 18) == (8, 64, 3)    # 61 runs: two rounds of 8
    assert tune_for(lib, 4, 1, 1 << 20) == (16, 32, 3)   # 241 runs: two rounds of 16
    assert tune_for(lib, 2, 1, 1 << 22) == (32, 32, 3)   # 964 runs: two rounds of 32
    assert tune_for(lib, 4, 1, 1 << 24) == (16, 32, 3)   # 3856 runs: three rounds of 16
    assert tune_for(lib, 2, 1, 1 << 27) == (32, 32, 3)
    assert lib.gms_rounds(0, 0, 1 << 24) == 3


def test_rounds_follow_the_fan_in(lib):
    try:
        assert lib.gms_rounds(0, 0, 1 << 28) == 3  # 8192 * 32^3 = 2^28
        assert lib.gms_set_tune(16, 32, 1) == GMS_OK
        assert lib.gms_rounds(0, 0, 1 << 28) == 4  # 8192 * 16^4 >= 2^28 > 8192 * 16^3
        assert lib.gms_set_tune(2, 32, 1) == GMS_OK
        assert lib.gms_rounds(0, 0, 1 << 28) == 15
    finally:
        lib.gms_clear_tune()


def test_pdl_switch(lib):
    """Programmatic dependent launch is on by default and switchable."""
    try:
        assert lib.gms_get_pdl() == 1
        assert lib.gms_set_pdl(0) == GMS_OK
        assert lib.gms_get_pdl() == 0
        assert lib.gms_set_pdl(2) == GMS_ERR_INVALID
        assert lib.gms_get_pdl() == 0
    finally:
        lib.gms_set_pdl(1)
    assert lib.gms_get_pdl() == 1


def test_argument_checks_before_device_work(lib):
    vp = ctypes.c_void_p
    assert lib.gms_sort_ws(9, 0, None, None, None, None, 10, None, 0, None) == GMS_ERR_INVALID
    assert b"dtype" in lib.gms_last_error()
    assert lib.gms_sort_ws(0, 2, None, None, None, None, 10, None, 0, None) == GMS_ERR_INVALID
    assert lib.gms_sort_ws(0, 0, None, None, None, None, 10, None, 0, None) == GMS_ERR_INVALID
    assert b"workspace" in lib.gms_last_error()
    assert lib.gms_sort_host_i32(None, None, 10, None) == GMS_ERR_INVALID
    assert b"null" in lib.gms_last_error()
    assert lib.gms_sort_host_i32(vp(16), vp(16), -1, None) == GMS_ERR_INVALID
    assert lib.gms_sort_host_i32_async(None, None, 10, None) == GMS_ERR_INVALID
    assert lib.gms_reserve(99, 0, 10, None) == GMS_ERR_INVALID
    assert lib.gms_reserve(0, 0, -1, None) == GMS_ERR_INVALID
    assert lib.gms_status_string(GMS_OK) == b"GMS_OK"
    assert lib.gms_status_string(12345) == b"GMS_ERR_UNKNOWN"


def test_workspace_size_grows_with_n(lib):
    sizes = [lib.gms_workspace_bytes(0, 0, n) for n in (1 << 16, 1 << 20, 1 << 24, 1 << 28)]
    assert sizes == sorted(sizes) and sizes[0] > 0
    # about N/B keys of block sample per level: well under the keys themselves
    assert sizes[-1] < (1 << 28) * 4 // 4
    assert lib.gms_workspace_bytes(0, 0, 0) == 0
    assert lib.gms_workspace_bytes(4, 1, 1 << 20) > lib.gms_workspace_bytes(0, 0, 1 << 20)


def test_strategy_choices(lib):
    """gms_set_tune_ex carries the splitter and base-case strategies (the
    reference's compile-time alternatives); gms_set_tune resets both."""
    q = [ctypes.c_int() for _ in range(5)]

    def get_ex():
        assert lib.gms_get_tune_ex(*[ctypes.byref(x) for x in q]) == GMS_OK
        return tuple(x.value for x in q)

    try:
        assert lib.gms_set_tune_ex(32, 32, 1, 1, 1) == GMS_OK
        assert get_ex() == (32, 32, 1, 1, 1)
        # the per-thread base case has 8704-key tiles: 2^28 keys still take 3 rounds
        assert lib.gms_rounds(0, 0, 1 << 28) == 3
        assert lib.gms_rounds(0, 0, 8704) == 0 and lib.gms_rounds(0, 0, 8705) == 1
        assert lib.gms_set_tune_ex(32, 32, 1, 2, 0) == GMS_ERR_INVALID
        assert b"split" in lib.gms_last_error()
        assert lib.gms_set_tune_ex(32, 32, 1, 0, 2) == GMS_ERR_INVALID
        assert b"base" in lib.gms_last_error()
        assert get_ex() == (32, 32, 1, 1, 1)
        assert lib.gms_set_tune(16, 32, 3) == GMS_OK
        assert get_ex() == (16, 32, 3, 0, 0)
        assert lib.gms_rounds(0, 0, 8193) == 1
    finally:
        lib.gms_clear_tune()


def test_segmented_argument_checks(lib):
    vp = ctypes.c_void_p
    # nothing to sort, or bad sizes, before any device work
    assert lib.gms_segmented_sort_i32(None, None, 0, None, 0, None) == GMS_OK
    assert lib.gms_segmented_sort_i32(None, None, -1, None, 1, None) == GMS_ERR_INVALID
    assert lib.gms_segmented_sort_u64(vp(16), vp(16), 10, None, 1, None) == GMS_ERR_INVALID
    assert b"null" in lib.gms_last_error()
    assert lib.gms_segmented_sort_kv_u64_i32(vp(16), None, vp(16), vp(16), 10, vp(16), 1, None) == GMS_ERR_INVALID
    assert lib.gms_segmented_sort_i32(vp(16), vp(16), 10, vp(16), 0, None) == GMS_ERR_INVALID
