"""GPU parity of the batched (segmented) sorts and of CUDA-graph replay.

Every segment of a batch must equal the oracle's sort of that segment
(std::sort; std::stable_sort by key with the payload for key/value batches)
and the result of one plain call on that segment alone (bit-exact).  Batches
mix every size class: arrays of one base tile or less (base case only), of
one merge round, and of two and three rounds bounded to the array.
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


@pytest.mark.parametrize("case", ["mixed", "tiny", "one", "empty_and_big", "equal", "all_classes", "three_rounds"])
def test_segmented_i32_matches_oracle(gms, oracle, case):
    lib = gms.load()
    rng = np.random.default_rng(sum(map(ord, case)))
    if case == "mixed":
        lengths = np.exp(rng.uniform(np.log(32), np.log(200000), 300)).astype(np.int64)
    elif case == "tiny":
        lengths = rng.integers(0, 40, 20000)
    elif case == "one":
        lengths = np.array([1_234_567])
    elif case == "empty_and_big":
        lengths = np.array([0, 0, 500_000, 0, 8192, 8193, 0, 1, 0])
    elif case == "all_classes":
        # base only, one round, two rounds (more than 32 tiles of 8192), at the class edges
        lengths = np.array([8192, 8193, 262144, 262145, 3, 2_000_003, 8191, 262143, 1, 700_000])
        lengths = np.concatenate([lengths, rng.integers(1, 600_000, 30)])
    elif case == "three_rounds":
        lengths = np.array([9_000_001, 17, 300_000, 0, 8_388_609])
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


@pytest.mark.parametrize("off", [[0, 60, 50, 100], [1, 60, 100], [0, 60, 99], [0, 60, 101]])
def test_segmented_bad_offsets_rejected(gms, off):
    lib = gms.load()
    keys = np.arange(100, dtype=np.int32)
    off = np.array(off, dtype=np.int64)  # not rising from 0 to n
    tin = torch.from_numpy(keys).cuda()
    tout = torch.empty_like(tin)
    toff = torch.from_numpy(off).cuda()
    rc = lib.gms_segmented_sort_i32(tin.data_ptr(), tout.data_ptr(), 100, toff.data_ptr(), len(off) - 1, _stream())
    assert rc == 1 and b"offsets" in lib.gms_last_error()


def test_segmented_u64_and_i64(gms, oracle):
    lib = gms.load()
    rng = np.random.default_rng(11)
    lengths = np.concatenate([[4096, 4097, 131072, 131073, 1, 0, 1_500_000],
                              np.exp(rng.uniform(np.log(16), np.log(400_000), 40)).astype(np.int64)])
    off = _offsets(lengths)
    n = int(off[-1])
    keys = oracle.gen_u64(n, 5)
    got = _gpu_segmented(lib, "gms_segmented_sort_u64", keys, off, view=np.int64)
    assert np.array_equal(got, oracle.segmented_sort(keys, off))
    ikeys = keys.view(np.int64)
    got = _gpu_segmented(lib, "gms_segmented_sort_i64", ikeys, off, view=np.int64)
    _check_segments(oracle, ikeys, off, got)


@pytest.mark.parametrize("kind", ["u64", "f32", "i32"])
def test_segmented_kv_stable(gms, oracle, kind):
    """Key/value batches: each array ordered by key, equal keys in input order
    (std::stable_sort per array), the payload moving with its key."""
    lib = gms.load()
    rng = np.random.default_rng(len(kind))
    lengths = np.concatenate([[4352, 4353, 139264, 139265, 1, 0, 900_001],
                              np.exp(rng.uniform(np.log(16), np.log(300_000), 30)).astype(np.int64)])
    off = _offsets(lengths)
    n = int(off[-1])
    if kind == "u64":
        keys = oracle.gen_u64(n, 6) % np.uint64(50_000)  # heavy ties: stability is visible
    elif kind == "f32":
        keys = oracle.gen_f32(n, 6)
    else:
        keys = (oracle.gen_i32(n, 0, 6) % 1000).astype(np.int32)
    vals = np.arange(n, dtype=np.int32)
    fn = {"u64": "gms_segmented_sort_kv_u64_i32", "f32": "gms_segmented_sort_kv_f32_i32",
          "i32": "gms_segmented_sort_kv_i32_i32"}[kind]
    view = np.int64 if kind == "u64" else np.int32
    ki = torch.from_numpy(keys.view(view).copy()).cuda()
    vi = torch.from_numpy(vals).cuda()
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    toff = torch.from_numpy(off).cuda()
    rc = getattr(lib, fn)(ki.data_ptr(), vi.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, toff.data_ptr(),
                          len(off) - 1, _stream())
    assert rc == 0, lib.gms_last_error()
    gk = ko.cpu().numpy().view(keys.dtype)
    gv = vo.cpu().numpy()
    if kind == "u64":
        wk, wv = oracle.segmented_sort_kv_u64(keys, vals, off)
        assert np.array_equal(gk, wk) and np.array_equal(gv, wv)
    else:
        for s in range(len(lengths)):
            a, b = off[s], off[s + 1]
            wk, wv = oracle.sort_kv(keys[a:b], vals[a:b])
            assert np.array_equal(gk[a:b].view(np.uint8), wk.view(np.uint8)) and np.array_equal(gv[a:b], wv), \
                f"segment {s}"
    assert np.array_equal(vi.cpu().numpy(), vals), "input payload must not be modified"


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
