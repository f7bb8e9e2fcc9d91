"""GPU parity of the batched (segmented) sort and of CUDA-graph replay.

Every segment of a batch must equal the oracle's std::sort of that segment and
the result of one plain gms_sort_i32 call on that segment alone (bit-exact).
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _offsets(lengths):
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    return off


def _gpu_segmented(lib, fn, keys, off, view=np.int32):
    tin = torch.from_numpy(keys.view(view).copy()).cuda()
    tout = torch.empty_like(tin)
    toff = torch.from_numpy(off).cuda()
    rc = getattr(lib, fn)(tin.data_ptr(), tout.data_ptr(), keys.size, toff.data_ptr(), len(off) - 1, _stream())
    assert rc == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(tin.cpu().numpy(), keys.view(view)), "input must not be modified"
    return tout.cpu().numpy().view(keys.dtype)


def _check_segments(oracle, keys, off, got):
    for s in range(len(off) - 1):
        a, b = off[s], off[s + 1]
        want = oracle.sort(keys[a:b])
        assert np.array_equal(got[a:b].view(np.uint8), want.view(np.uint8)), f"segment {s} [{a},{b})"


@pytest.mark.parametrize("case", ["mixed", "tiny", "one", "empty_and_big", "equal"])
def test_segmented_i32_matches_oracle(gms, oracle, case):
    lib = gms.load()
    rng = np.random.default_rng(hash(case) % 1000)
    if case == "mixed":
        lengths = np.exp(rng.uniform(np.log(32), np.log(200000), 300)).astype(np.int64)
    elif case == "tiny":
        lengths = rng.integers(0, 40, 20000)
    elif case == "one":
        lengths = np.array([1_234_567])
    elif case == "empty_and_big":
        lengths = np.array([0, 0, 500_000, 0, 8192, 8193, 0, 1, 0])
    else:
        lengths = rng.integers(1, 5000, 500)
    off = _offsets(lengths)
    n = int(off[-1])
    keys = oracle.gen_i32(n, 3 if case == "equal" else 6, 42)
    got = _gpu_segmented(lib, "gms_segmented_sort_i32", keys, off)
    _check_segments(oracle, keys, off, got)
    assert gms.device_status() == 0


def test_segmented_f32_total_order(gms, oracle):
    lib = gms.load()
    lengths = np.array([100, 0, 70_000, 3, 9000, 1])
    off = _offsets(lengths)
    keys = oracle.gen_f32(int(off[-1]), 9)
    got = _gpu_segmented(lib, "gms_segmented_sort_f32", keys, off)
    _check_segments(oracle, keys, off, got)


def test_segmented_equals_plain_calls(gms, oracle):
    """Batched result == one plain multimergesort call per array."""
    lib = gms.load()
    rng = np.random.default_rng(3)
    lengths = np.exp(rng.uniform(np.log(32), np.log(300000), 60)).astype(np.int64)
    off = _offsets(lengths)
    keys = oracle.gen_i32(int(off[-1]), 0, 17)
    got = _gpu_segmented(lib, "gms_segmented_sort_i32", keys, off)
    for s in range(len(lengths)):
        a, b = off[s], off[s + 1]
        tin = torch.from_numpy(keys[a:b].copy()).cuda()
        tout = torch.empty_like(tin)
        assert lib.gms_sort_i32(tin.data_ptr(), tout.data_ptr(), b - a, 0, _stream()) == 0
        assert np.array_equal(tout.cpu().numpy(), got[a:b]), f"segment {s}"


def test_segmented_bad_offsets_flagged(gms):
    lib = gms.load()
    keys = np.arange(100, dtype=np.int32)
    off = np.array([0, 60, 50, 100], dtype=np.int64)  # not monotone
    tin = torch.from_numpy(keys).cuda()
    tout = torch.empty_like(tin)
    toff = torch.from_numpy(off).cuda()
    assert lib.gms_segmented_sort_i32(tin.data_ptr(), tout.data_ptr(), 100, toff.data_ptr(), 3, _stream()) == 0
    assert gms.device_status() & 8


def test_graph_replay_sort(gms, oracle):
    lib = gms.load()
    n = 3_000_001
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    tin = torch.empty(n, dtype=torch.int32, device="cuda")
    tout = torch.empty_like(tin)
    g = ctypes.c_void_p()
    with torch.cuda.stream(s):
        tin.copy_(torch.from_numpy(oracle.gen_i32(n, 0, 1)))
        s.synchronize()
        assert lib.gms_graph_create_sort_i32(tin.data_ptr(), tout.data_ptr(), n, sp, ctypes.byref(g)) == 0, \
            lib.gms_last_error()
        for seed in (5, 6):
            a = oracle.gen_i32(n, 6, seed)
            tin.copy_(torch.from_numpy(a))
            assert lib.gms_graph_launch(g, sp) == 0
            s.synchronize()
            assert np.array_equal(tout.cpu().numpy(), oracle.sort(a)), f"seed {seed}"
    assert lib.gms_graph_destroy(g) == 0


def test_graph_replay_segmented(gms, oracle):
    lib = gms.load()
    rng = np.random.default_rng(8)
    lengths = np.exp(rng.uniform(np.log(32), np.log(100000), 200)).astype(np.int64)
    off = _offsets(lengths)
    n = int(off[-1])
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    with torch.cuda.stream(s):
        tin = torch.from_numpy(oracle.gen_i32(n, 0, 2)).cuda()
        tout = torch.empty_like(tin)
        toff = torch.from_numpy(off).cuda()
        s.synchronize()
        g = ctypes.c_void_p()
        assert lib.gms_graph_create_segmented_i32(tin.data_ptr(), tout.data_ptr(), n, toff.data_ptr(), len(lengths), sp,
                                                  ctypes.byref(g)) == 0, lib.gms_last_error()
        a = oracle.gen_i32(n, 4, 77)
        tin.copy_(torch.from_numpy(a))
        assert lib.gms_graph_launch(g, sp) == 0
        s.synchronize()
        _check_segments(oracle, a, off, tout.cpu().numpy())
        assert lib.gms_graph_destroy(g) == 0
