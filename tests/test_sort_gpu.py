"""GPU parity: the sm_103a library, called through its C ABI, against the oracle.

Integer, float (total order) and key/value results must be bit-identical to
std::sort / std::stable_sort (oracle/oracle.cpp).  The reference-generated
golden set (tests/golden/ref_random_list.npz: the reference's own input
generator and its selection-sort checker) is replayed first.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SIGNED = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64, np.dtype(np.float32): np.int32,
          np.dtype(np.float64): np.int64, np.dtype(np.int32): np.int32, np.dtype(np.int64): np.int64}
SUFFIX = {np.dtype(np.int32): "i32", np.dtype(np.uint32): "u32", np.dtype(np.float32): "f32",
          np.dtype(np.int64): "i64", np.dtype(np.uint64): "u64", np.dtype(np.float64): "f64"}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(SIGNED[a.dtype])).cuda()


def from_dev(t, dtype):
    return t.cpu().numpy().view(dtype)


def stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def gpu_sort(gms, a):
    lib = gms.load()
    tin = to_dev(a)
    tout = torch.empty_like(tin)
    fn = getattr(lib, "gms_sort_" + SUFFIX[a.dtype])
    st = fn(tin.data_ptr(), tout.data_ptr(), a.size, 0, stream())
    assert st == 0, lib.gms_last_error()
    assert gms.device_status() == 0
    return from_dev(tout, a.dtype)


def gpu_sort_kv(gms, k, v):
    lib = gms.load()
    ki, vi = to_dev(k), to_dev(v.astype(np.int32))
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    fn = getattr(lib, f"gms_sort_kv_{SUFFIX[k.dtype]}_i32")
    st = fn(ki.data_ptr(), vi.data_ptr(), ko.data_ptr(), vo.data_ptr(), k.size, 0, stream())
    assert st == 0, lib.gms_last_error()
    assert gms.device_status() == 0
    return from_dev(ko, k.dtype), from_dev(vo, np.int32)


def assert_same(got, want, what=""):
    if not np.array_equal(got.view(SIGNED[got.dtype]), want.view(SIGNED[want.dtype])):
        d = np.nonzero(got.view(SIGNED[got.dtype]) != want.view(SIGNED[want.dtype]))[0]
        raise AssertionError(f"{what}: {d.size} mismatches, first at {d[0]}: got {got[d[0]]} want {want[d[0]]}")


# ---------------------------------------------------------------------------
def test_reference_golden_inputs(gms, golden):
    """The reference's own test inputs, sorted as its checker sorts them."""
    for n, seed in [tuple(int(x) for x in c) for c in golden["cases"]]:
        got = gpu_sort(gms, golden[f"in_{n}_{seed}"])
        assert_same(got, golden[f"sorted_{n}_{seed}"], f"n={n} seed={seed}")


def test_tile_sort_matches_square_sort_golden(gms, golden):
    """squareSort contract with the reference's M=1024 tiles (and tail)."""
    lib = gms.load()
    for n, seed in [tuple(int(x) for x in c) for c in golden["cases"]]:
        if n == 0:
            continue
        t = to_dev(golden[f"in_{n}_{seed}"])
        assert lib.gms_tile_sort_i32(t.data_ptr(), n, 1024, stream()) == 0
        assert_same(from_dev(t, np.int32), golden[f"tiles1024_{n}_{seed}"], f"n={n}")


@pytest.mark.parametrize("tile", [1, 2, 17, 1000, 4096, 8703, 8704])
def test_tile_sort_tiles(gms, oracle, tile):
    lib = gms.load()
    a = oracle.gen_i32(50001, 6, tile)
    t = to_dev(a)
    assert lib.gms_tile_sort_i32(t.data_ptr(), a.size, tile, stream()) == 0
    assert_same(from_dev(t, np.int32), oracle.tile_sort(a, tile), f"tile={tile}")


SIZES = [0, 1, 2, 3, 31, 100, 1023, 8703, 8704, 8705, 17409, 100000, 278528, 278529, 1000003, 3 * 278528 + 17]


@pytest.mark.parametrize("n", SIZES)
def test_sort_i32_sizes(gms, oracle, n):
    a = oracle.gen_i32(n, 6, 1000 + n)
    assert_same(gpu_sort(gms, a), oracle.sort(a), f"n={n}")


@pytest.mark.parametrize("dist", range(7))
def test_sort_i32_distributions(gms, oracle, dist):
    n = (1 << 22) + 12345
    a = oracle.gen_i32(n, dist, 77)
    assert_same(gpu_sort(gms, a), oracle.sort(a), f"dist={dist}")


def test_sort_i32_two_rounds(gms, oracle):
    n = 9_000_001  # 2 merge rounds, recursive sample merge
    a = oracle.gen_i32(n, 6, 5)
    assert_same(gpu_sort(gms, a), oracle.sort(a))


# Buffers that start inside a 16-byte line: the merged tiles are stored with
# 16-byte accesses between single keys at both ends of every tile, so output
# (and input) pointers 1..E-1 keys past a 16-byte boundary must give the same
# bits.  The keys around the sorted range must stay untouched.
@pytest.mark.parametrize("dtype,shift", [(np.int32, 1), (np.int32, 3), (np.uint32, 2), (np.int64, 1),
                                         (np.float32, 1)])
def test_sort_unaligned_buffers(gms, oracle, dtype, shift):
    lib = gms.load()
    rng = np.random.default_rng(shift * 10 + np.dtype(dtype).itemsize)
    for n in [37, 8192 + 5, 300_007, 2_000_011]:
        if dtype == np.float32:
            a = oracle.gen_f32(n, n)
        else:
            info = np.iinfo(dtype)
            a = rng.integers(info.min, info.max, n, dtype=dtype, endpoint=True)
        tin_all = to_dev(np.concatenate([np.zeros(shift + 2, dtype), a]))
        tout_all = torch.full((n + shift + 2,), 7, dtype=tin_all.dtype, device="cuda")
        tin, tout = tin_all[shift + 2:], tout_all[shift:shift + n]
        fn = getattr(lib, "gms_sort_" + SUFFIX[np.dtype(dtype)])
        assert fn(tin.data_ptr(), tout.data_ptr(), n, 0, stream()) == 0, lib.gms_last_error()
        assert gms.device_status() == 0
        got = from_dev(tout_all, dtype)
        assert_same(got[shift:shift + n], oracle.sort(a), f"{dtype} shift={shift} n={n}")
        assert np.all(got.view(SIGNED[got.dtype])[:shift] == 7) and np.all(got.view(SIGNED[got.dtype])[shift + n:] == 7)


@pytest.mark.parametrize("dtype", [np.uint32, np.int64, np.uint64])
def test_sort_integer_dtypes(gms, oracle, dtype):
    rng = np.random.default_rng(9)
    info = np.iinfo(dtype)
    for n in [5, 8705, 300001, 2_500_003]:
        a = rng.integers(info.min, info.max, n, dtype=dtype, endpoint=True)
        assert_same(gpu_sort(gms, a), oracle.sort(a), f"{dtype} n={n}")


def test_sort_f32_total_order(gms, oracle):
    for n in [7, 8705, 1_000_003]:
        a = oracle.gen_f32(n, 31 + n)
        assert_same(gpu_sort(gms, a), oracle.sort(a), f"n={n}")


def test_sort_f64_total_order(gms, oracle):
    a = oracle.gen_f32(700001, 3).astype(np.float64)
    a[::1000] = -0.0
    bits = a.view(np.uint64)
    bits[5::997] = np.uint64(0xFFF8000000000123)  # negative NaN with payload
    assert_same(gpu_sort(gms, a), oracle.sort(a))


def test_full_key_range_extremes(gms, oracle):
    """No sentinel: INT_MAX / INT_MIN (the reference's MAXVAL) sort like any key."""
    rng = np.random.default_rng(4)
    a = rng.choice(np.array([2**31 - 1, -2**31, 0, -1, 1, 2**31 - 2], dtype=np.int32), 300007)
    assert_same(gpu_sort(gms, a), oracle.sort(a))
    b = rng.choice(np.array([2**64 - 1, 0, 2**63, 2**63 - 1], dtype=np.uint64), 100003)
    assert_same(gpu_sort(gms, b), oracle.sort(b))


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 100, 8705, 300001, 2_000_003])
def test_kv_u64_stable(gms, oracle, n):
    k = oracle.gen_u64(n, 17 + n)
    k[::3] = k[0]  # many ties: stability is visible in the payload
    v = np.arange(n, dtype=np.int32)
    gk, gv = gpu_sort_kv(gms, k, v)
    ok, ov = oracle.sort_kv(k, v)
    assert_same(gk, ok, "keys")
    assert_same(gv, ov, "payload")


@pytest.mark.parametrize("dtype", [np.int32, np.uint32, np.float32, np.int64, np.float64])
def test_kv_other_dtypes(gms, oracle, dtype):
    rng = np.random.default_rng(12)
    n = 400009
    if dtype == np.float32:
        k = oracle.gen_f32(n, 5)
    elif dtype == np.float64:
        k = oracle.gen_f32(n, 6).astype(np.float64)
    else:
        k = rng.integers(-50 if np.dtype(dtype).kind == "i" else 0, 50, n).astype(dtype)
    v = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
    gk, gv = gpu_sort_kv(gms, k, v)
    ok, ov = oracle.sort_kv(k, v)
    assert_same(gk, ok, "keys")
    assert_same(gv, ov, "payload")


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("run_len,k", [(1, 2), (1, 32), (7, 3), (100, 32), (1000, 32), (8704, 32), (5000, 7),
                                       (100000, 4)])
def test_merge_level(gms, oracle, run_len, k):
    lib = gms.load()
    n = 600011
    a = oracle.tile_sort(oracle.gen_i32(n, 4 if k == 7 else 6, run_len), run_len)
    t = to_dev(a)
    o = torch.empty_like(t)
    assert lib.gms_merge_level_i32(t.data_ptr(), o.data_ptr(), n, run_len, k, stream()) == 0, lib.gms_last_error()
    assert gms.device_status() == 0
    assert_same(from_dev(o, np.int32), oracle.merge_level(a, run_len, k), f"L={run_len} k={k}")
    assert_same(from_dev(t, np.int32), a, "input untouched")


def test_merge_level_u64(gms, oracle):
    lib = gms.load()
    n, L, k = 400003, 3001, 16
    a = np.sort(oracle.gen_u64(n, 1).reshape(-1)[: n])
    a = oracle.tile_sort(oracle.gen_u64(n, 2), L)
    t = to_dev(a)
    o = torch.empty_like(t)
    assert lib.gms_merge_level_u64(t.data_ptr(), o.data_ptr(), n, L, k, stream()) == 0
    assert_same(from_dev(o, np.uint64), oracle.merge_level(a, L, k))


@pytest.mark.parametrize("size,k", [(1000, 8), (50000, 32), (100, 3)])
def test_find_partitions(gms, oracle, size, k):
    lib = gms.load()
    task = oracle.tile_sort(oracle.gen_i32(size * k - 5, 4, size), size)
    mergers = 13
    ranks = np.array([m * task.size // mergers for m in range(mergers + 1)] + [1, task.size - 1], dtype=np.int64)
    tt, tr = to_dev(task), torch.from_numpy(ranks).cuda()
    out = torch.empty((ranks.size, k), dtype=torch.int64, device="cuda")
    st = lib.gms_find_partitions_i32(tt.data_ptr(), size, k, task.size, tr.data_ptr(), ranks.size, out.data_ptr(),
                                     stream())
    assert st == 0, lib.gms_last_error()
    assert np.array_equal(out.cpu().numpy(), oracle.find_partitions(task, size, k, ranks))


# ---------------------------------------------------------------------------
def test_deterministic_repeats(gms, oracle):
    a = oracle.gen_i32(2_000_003, 5, 3)
    first = gpu_sort(gms, a)
    for _ in range(3):
        assert_same(gpu_sort(gms, a), first)


def test_programmatic_launch_on_off_and_two_streams(gms, oracle):
    """Sorts launched with programmatic dependent launch (the default) and in
    plain stream order give the oracle's result, also while two streams sort
    at the same time (each stream's kernels wait only for their own
    predecessors)."""
    lib = gms.load()
    sizes = (300_007, 2_000_003, 9_000_001)
    inputs = [oracle.gen_i32(n, d, 40 + d) for d, n in enumerate(sizes)]
    wants = [oracle.sort(a) for a in inputs]
    try:
        for pdl in (1, 0):
            assert lib.gms_set_pdl(pdl) == 0
            for a, want in zip(inputs, wants):
                assert_same(gpu_sort(gms, a), want, f"pdl={pdl} n={a.size}")
        assert lib.gms_set_pdl(1) == 0
        streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        tins = [to_dev(a) for a in inputs[1:]]
        touts = [torch.empty_like(t) for t in tins]
        torch.cuda.synchronize()
        for rep in range(3):
            for s, tin, tout in zip(streams, tins, touts):
                with torch.cuda.stream(s):
                    tin_c = tin.clone()
                    st = lib.gms_sort_i32(tin_c.data_ptr(), tout.data_ptr(), tin.numel(), 0,
                                          ctypes.c_void_p(s.cuda_stream))
                    assert st == 0, lib.gms_last_error()
            torch.cuda.synchronize()
            for tout, want in zip(touts, wants[1:]):
                assert_same(from_dev(tout, np.int32), want, f"two streams, rep {rep}")
    finally:
        lib.gms_set_pdl(1)


def test_host_entry_point(gms, oracle):
    lib = gms.load()
    a = oracle.gen_i32(1_000_003, 0, 8)
    hin = torch.from_numpy(a.copy()).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), a.size, stream()) == 0
    assert_same(hout.numpy(), oracle.sort(a))


def test_invalid_arguments(gms):
    lib = gms.load()
    t = torch.zeros(16, dtype=torch.int32, device="cuda")
    assert lib.gms_sort_i32(t.data_ptr(), t.data_ptr(), -1, 0, stream()) == 1
    assert lib.gms_sort_i32(None, t.data_ptr(), 5, 0, stream()) == 1
    assert lib.gms_merge_level_i32(t.data_ptr(), t.data_ptr(), 16, 4, 1, stream()) == 1
    assert lib.gms_merge_level_i32(t.data_ptr(), t.data_ptr(), 16, 4, 33, stream()) == 1
    assert lib.gms_tile_sort_i32(t.data_ptr(), 16, 0, stream()) == 1
    assert lib.gms_tile_sort_i32(t.data_ptr(), 16, 8705, stream()) == 1
    assert b"n" in lib.gms_last_error() or lib.gms_last_error() != b""
    assert lib.gms_sort_i32(t.data_ptr(), t.data_ptr(), 0, 0, stream()) == 0


# ---------------------------------------------------------------------------
# Tuning: other fan-ins, sample block sizes and every staging mode (one bulk
# copy per segment, the same with persistent CTAs, 16-byte copies by every
# warp, plain loads) must give the same bits.
TUNES = [(32, 32, 0), (2, 32, 1), (3, 16, 1), (7, 64, 1), (16, 8, 1), (32, 96, 1), (5, 100, 0), (32, 17, 1),
         (32, 32, 2), (16, 8, 2), (3, 64, 2), (32, 32, 3), (16, 8, 3), (2, 32, 3), (7, 64, 3)]


@pytest.fixture
def tuned(gms):
    lib = gms.load()
    yield lib
    assert lib.gms_clear_tune() == 0


@pytest.mark.parametrize("k,b,bulk", TUNES)
def test_tune_variants(gms, oracle, tuned, k, b, bulk):
    lib = tuned
    assert lib.gms_set_tune(k, b, bulk) == 0
    for n, dist in [(8705, 6), (300001, 0), (1_234_567, 4), (2_000_003, 1), (1_500_001, 3)]:
        a = oracle.gen_i32(n, dist, 7 * k + b)
        assert_same(gpu_sort(gms, a), oracle.sort(a), f"k={k} b={b} bulk={bulk} n={n} dist={dist}")
    k64 = oracle.gen_u64(700001, k)
    v = np.arange(k64.size, dtype=np.int32)
    k64[::2] = k64[1]
    gk, gv = gpu_sort_kv(gms, k64, v)
    ok_, ov_ = oracle.sort_kv(k64, v)
    assert_same(gk, ok_, "kv keys")
    assert_same(gv, ov_, "kv payload")


# The strategy switches (the reference's compile-time alternatives): the
# direct findPartitions-style splitter and the per-thread base case, alone and
# together, on 32- and 64-bit keys, keys only and with a payload, and batched.
@pytest.mark.parametrize("split,base", [(1, 0), (0, 1), (1, 1)])
def test_strategy_variants(gms, oracle, tuned, split, base):
    lib = tuned
    assert lib.gms_set_tune_ex(32, 32, 1, split, base) == 0, lib.gms_last_error()
    for n, dist in [(8704, 0), (8705, 6), (300001, 0), (2_500_001, 4), (3_000_003, 5)]:
        a = oracle.gen_i32(n, dist, 3 + split + 2 * base)
        assert_same(gpu_sort(gms, a), oracle.sort(a), f"split={split} base={base} n={n} dist={dist}")
    u = oracle.gen_u64(1_000_003, 9)
    assert_same(gpu_sort(gms, u), oracle.sort(u), "u64")
    k64 = oracle.gen_u64(700001, 4)
    v = np.arange(k64.size, dtype=np.int32)
    k64[::3] = k64[1]
    gk, gv = gpu_sort_kv(gms, k64, v)
    ok_, ov_ = oracle.sort_kv(k64, v)
    assert_same(gk, ok_, "kv keys")
    assert_same(gv, ov_, "kv payload")
    # a batch of arrays under the same strategies
    lengths = np.array([1, 8704, 8705, 300000, 0, 4000, 1_200_000], dtype=np.int64)
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    keys = oracle.gen_i32(int(off[-1]), 0, 5)
    tin = torch.from_numpy(keys).cuda()
    tout = torch.empty_like(tin)
    toff = torch.from_numpy(off).cuda()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.gms_segmented_sort_i32(tin.data_ptr(), tout.data_ptr(), keys.size, toff.data_ptr(), len(lengths),
                                      st) == 0, lib.gms_last_error()
    assert_same(tout.cpu().numpy(), oracle.segmented_sort(keys, off), "batched")


def test_tune_rejects_bad_values(gms, tuned):
    lib = tuned
    assert lib.gms_set_tune(1, 32, 1) == 1
    assert lib.gms_set_tune(33, 32, 1) == 1
    assert lib.gms_set_tune(32, 0, 1) == 1
    assert lib.gms_set_tune(32, 300, 1) == 1  # 4080/300 - 32 < 1
    assert lib.gms_set_tune(32, 128, 1) == 1  # 4080/128 - 32 < 1


# Explicit workspace: same bits as the cached-scratch sort, for keys-only and
# key/value dtypes; too-small and misaligned workspaces are refused.
@pytest.mark.parametrize("dtype,kv", [(0, 0), (2, 0), (4, 0), (5, 0), (0, 1), (4, 1), (2, 1)])
def test_sort_with_explicit_workspace(gms, oracle, dtype, kv):
    lib = gms.load()
    n = 1_234_567
    np_t = {0: np.int32, 2: np.float32, 4: np.uint64, 5: np.float64}[dtype]
    if dtype == 0:
        keys = oracle.gen_i32(n, 6, 5)
    elif dtype == 2:
        keys = oracle.gen_f32(n, 5)
    elif dtype == 4:
        keys = oracle.gen_u64(n, 5)
        keys[::3] = keys[1]
    else:
        keys = oracle.gen_f32(n, 6).astype(np.float64)
    vals = np.arange(n, dtype=np.int32)
    view = np.int64 if keys.itemsize == 8 else np.int32
    kin = torch.from_numpy(keys.view(view).copy()).cuda()
    kout = torch.empty_like(kin)
    vin = torch.from_numpy(vals).cuda() if kv else None
    vout = torch.empty_like(vin) if kv else None
    need = lib.gms_workspace_bytes(dtype, kv, n)
    assert need > 0
    ws = torch.empty(need + 256, dtype=torch.uint8, device="cuda")
    base = ws.data_ptr() + (-ws.data_ptr()) % 256
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    assert lib.gms_sort_ws(dtype, kv, kin.data_ptr(), vp(vin), kout.data_ptr(), vp(vout), n, base, need - 8, st) == 1
    assert lib.gms_sort_ws(dtype, kv, kin.data_ptr(), vp(vin), kout.data_ptr(), vp(vout), n, base + 8, need, st) == 1
    rc = lib.gms_sort_ws(dtype, kv, kin.data_ptr(), vp(vin), kout.data_ptr(), vp(vout), n, base, need, st)
    assert rc == 0, lib.gms_last_error()
    flag = ctypes.c_int(-1)
    assert lib.gms_workspace_status(base, st, ctypes.byref(flag)) == 0 and flag.value == 0
    got = kout.cpu().numpy().view(np_t)
    if kv:
        wk, wv = oracle.sort_kv(keys, vals)
        assert np.array_equal(got.view(np.uint8), wk.view(np.uint8))
        assert np.array_equal(vout.cpu().numpy(), wv)
    else:
        assert np.array_equal(got.view(np.uint8), oracle.sort(keys).view(np.uint8))


# Host-to-host sorts: the synchronous call (input copied in pieces that the base
# case sorts as they land) and the pipelined call with two sorts in flight.
def test_host_sort_pipelined(gms, oracle):
    lib = gms.load()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # the last two sizes sort their first merge round piece by piece
    for n in (1, 8191, 8193, 3 * 8192 + 5, 1_000_003, (1 << 22) + 12345, (1 << 25) + 5):
        a = oracle.gen_i32(n, 6, n)
        hin = torch.from_numpy(a).pin_memory()
        hout = torch.empty_like(hin).pin_memory()
        assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, st) == 0, lib.gms_last_error()
        assert np.array_equal(hout.numpy(), oracle.sort(a)), n
        pageable = np.empty(n, dtype=np.int32)  # pageable output memory
        assert lib.gms_sort_host_i32(hin.data_ptr(), pageable.ctypes.data, n, st) == 0, lib.gms_last_error()
        assert np.array_equal(pageable, oracle.sort(a)), n
        inplace = torch.from_numpy(a.copy()).pin_memory()  # output over the input
        assert lib.gms_sort_host_i32(inplace.data_ptr(), inplace.data_ptr(), n, st) == 0
        assert np.array_equal(inplace.numpy(), oracle.sort(a)), n
    n = 2_500_001
    ins = [oracle.gen_i32(n, d, 30 + d) for d in range(5)]
    hins = [torch.from_numpy(x).pin_memory() for x in ins]
    houts = [torch.empty_like(h).pin_memory() for h in hins]
    for h, o in zip(hins, houts):
        assert lib.gms_sort_host_i32_async(h.data_ptr(), o.data_ptr(), n, st) == 0, lib.gms_last_error()
    assert lib.gms_host_sync(st) == 0
    for x, o in zip(ins, houts):
        assert np.array_equal(o.numpy(), oracle.sort(x))
    # a larger call after smaller ones regrows the pipeline's buffers
    big = oracle.gen_i32(4_000_000, 0, 99)
    hb = torch.from_numpy(big).pin_memory()
    ob = torch.empty_like(hb).pin_memory()
    assert lib.gms_sort_host_i32_async(hb.data_ptr(), ob.data_ptr(), big.size, st) == 0
    assert lib.gms_host_sync(st) == 0
    assert np.array_equal(ob.numpy(), oracle.sort(big))


def test_host_sort_async_mixed_sizes(gms, oracle):
    # asynchronous calls of growing and shrinking sizes in flight together, so
    # each buffer set of the pipeline grows while the others are busy, with a
    # synchronous call (which takes the first buffer set) in between
    lib = gms.load()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sizes = [100_000, 3_000_017, 50_001, 2_000_000, 6_000_011, 10, 1_000_003, 4_500_000]
    ins = [oracle.gen_i32(n, i % 6, 70 + i) for i, n in enumerate(sizes)]
    hins = [torch.from_numpy(x).pin_memory() for x in ins]
    houts = [torch.empty_like(h).pin_memory() for h in hins]
    for i, (h, o) in enumerate(zip(hins, houts)):
        if i == 4:
            assert lib.gms_sort_host_i32(h.data_ptr(), o.data_ptr(), sizes[i], st) == 0, lib.gms_last_error()
        else:
            assert lib.gms_sort_host_i32_async(h.data_ptr(), o.data_ptr(), sizes[i], st) == 0, lib.gms_last_error()
    assert lib.gms_host_sync(st) == 0
    for x, o in zip(ins, houts):
        assert np.array_equal(o.numpy(), oracle.sort(x)), x.size


# Beyond 2^31 keys (64-bit sizes and offsets everywhere): at this size the
# result is checked through size-independent properties -- sortedness, and the
# multiset through order-independent sums -- rather than against the oracle.
def test_sort_i32_beyond_2p31_properties(gms):
    lib = gms.load()
    n = (1 << 31) + 1001
    free, _ = torch.cuda.mem_get_info()
    if free < 24 * (1 << 30):
        pytest.skip("needs ~24 GB of free device memory")
    g = torch.Generator(device="cuda")
    g.manual_seed(123)
    keys = torch.randint(-(2**31), 2**31 - 1, (n,), dtype=torch.int32, device="cuda", generator=g)
    keys[:: 1 << 20] = 2**31 - 1  # full range, heavy values at the ends
    keys[7 :: 1 << 21] = -(2**31)

    def sums(t):  # in chunks: a 2^31-element int64 temporary would need 17 GB
        acc = [0, 0, 0]
        for c in torch.split(t, 1 << 28):
            x = c.to(torch.int64)
            acc[0] += int(x.sum())
            acc[1] += int(((x * x) % 1000000007).sum())
            acc[2] += int((x * 2654435761 % 1000003).sum())
        return tuple(acc)

    before = sums(keys)
    out = torch.empty_like(keys)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.gms_sort_i32(keys.data_ptr(), out.data_ptr(), n, 0, st) == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    assert gms.device_status() == 0
    assert bool((out[1:] >= out[:-1]).all()), "not sorted"
    assert sums(out) == before, "not a permutation of the input"
    assert int(out[0]) == -(2**31) and int(out[-1]) == 2**31 - 1
