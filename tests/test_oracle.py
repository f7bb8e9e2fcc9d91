"""The oracle pinned against the reference's own routines (CPU only).

tests/golden/ref_random_list.npz was produced by the reference's own code
(create_random_list after srand(seed), src/buildData.h:54-65 and
src/testMM.cu:156; selection_sort<int,host_cmp>, src/testMM.cu:308-320; and
the per-tile selection sort test_squareSort checks the base case with,
src/testMM.cu:264-269), built from its sources by oracle/Makefile and run by
tests/golden/make_golden.py.
"""
import numpy as np
import pytest


def _cases(golden):
    return [tuple(int(x) for x in c) for c in golden["cases"]]


def test_generator_matches_reference(oracle, golden):
    for n, seed in _cases(golden):
        assert np.array_equal(oracle.ref_random_list(n, seed), golden[f"in_{n}_{seed}"]), (n, seed)


def test_sort_matches_reference_selection_sort(oracle, golden):
    for n, seed in _cases(golden):
        assert np.array_equal(oracle.sort(golden[f"in_{n}_{seed}"]), golden[f"sorted_{n}_{seed}"]), (n, seed)


def test_tile_sort_matches_reference_square_sort_check(oracle, golden):
    for n, seed in _cases(golden):
        got = oracle.tile_sort(golden[f"in_{n}_{seed}"], 1024)
        assert np.array_equal(got, golden[f"tiles1024_{n}_{seed}"]), (n, seed)


def test_selection_sort_restatement(oracle, golden):
    for n, seed in _cases(golden)[:10]:
        assert np.array_equal(oracle.selection_sort(golden[f"in_{n}_{seed}"]), golden[f"sorted_{n}_{seed}"])


@pytest.mark.parametrize("dtype", [np.int32, np.uint32, np.int64, np.uint64])
def test_sort_integer_matches_numpy(oracle, dtype):
    rng = np.random.default_rng(1)
    info = np.iinfo(dtype)
    a = rng.integers(info.min, info.max, 10007, dtype=dtype, endpoint=True)
    assert np.array_equal(oracle.sort(a), np.sort(a))


def _total_order_key32(a):
    b = a.view(np.uint32)
    return np.where(b & 0x80000000, ~b, b | 0x80000000)


def test_float_total_order(oracle):
    a = oracle.gen_f32(200003, 5)
    assert np.isnan(a).sum() > 0 and (a == 0).sum() > 0
    s = oracle.sort(a)
    keys = _total_order_key32(s)
    assert np.all(keys[1:] >= keys[:-1])
    # -0.0 before +0.0, negative NaN first, positive NaN last
    z = np.where(s == 0)[0]
    assert np.signbit(s[z[0]]) and not np.signbit(s[z[-1]])
    assert np.isnan(s[-1]) and not np.signbit(s[-1])
    assert np.array_equal(np.sort(keys), keys)


def test_kv_is_stable_sort_by_key(oracle):
    rng = np.random.default_rng(2)
    k = rng.integers(0, 50, 20000).astype(np.uint64)
    v = np.arange(k.size, dtype=np.int32)
    sk, sv = oracle.sort_kv(k, v)
    order = np.argsort(k, kind="stable")
    assert np.array_equal(sk, k[order]) and np.array_equal(sv, v[order])


def test_merge_level_and_partitions(oracle):
    rng = np.random.default_rng(3)
    L, K = 100, 5
    a = rng.integers(0, 30, 1234).astype(np.int32)
    runs = oracle.tile_sort(a, L)
    merged = oracle.merge_level(runs, L, K)
    for g in range(0, a.size, L * K):
        assert np.array_equal(merged[g:g + L * K], np.sort(runs[g:g + L * K], kind="stable"))
    task = runs[:L * K]
    ranks = np.array([0, 1, 77, 250, 499, 500], dtype=np.int64)
    co = oracle.find_partitions(task, L, K, ranks)
    assert np.array_equal(co.sum(axis=1), ranks)
    # brute force: stable order tags
    tags = np.repeat(np.arange(K), L)
    order = np.argsort(task, kind="stable")
    for q, r in enumerate(ranks):
        assert np.array_equal(np.bincount(tags[order[:r]], minlength=K), co[q])


def test_generators_deterministic(oracle):
    for d in range(7):
        x = oracle.gen_i32(5000, d, 11)
        y = oracle.gen_i32(5000, d, 11)
        assert np.array_equal(x, y)
    assert np.all(oracle.gen_i32(1000, 3, 1) == 42)
    assert len(np.unique(oracle.gen_i32(100000, 4, 1))) <= 16
    s = oracle.gen_i32(10000, 1, 1)
    assert np.all(s[1:] >= s[:-1])
    r = oracle.gen_i32(10000, 2, 1)
    assert np.all(r[1:] <= r[:-1])
