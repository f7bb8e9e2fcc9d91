"""CPU check of the round/tile index arithmetic (tests/plan_model.py mirrors
gms_sort.cuh and the splitter/tile kernels): every input distribution sorts
stably and no tile at any recursion level exceeds the shared-memory capacity."""
import numpy as np
import pytest

from plan_model import Geometry, model_sort


def dists(rng, n):
    yield "uniform", rng.integers(0, 2**31 - 1, n)
    yield "sorted", np.sort(rng.integers(0, 2**31 - 1, n))
    yield "reverse", np.sort(rng.integers(0, 2**31 - 1, n))[::-1].copy()
    yield "equal", np.full(n, 42)
    yield "sixteen", rng.choice(rng.integers(0, 2**31 - 1, 16), n)
    yield "zipf", np.minimum(rng.zipf(1.2, n), 2**20)
    yield "sawtooth", np.arange(n) % 97


@pytest.mark.parametrize("cap,k,b", [(40, 4, 2), (64, 4, 4), (96, 8, 4), (136, 32, 4)])
def test_tiles_fit_and_sort_is_stable(cap, k, b):
    geo = Geometry(cap, k, b)
    rng = np.random.default_rng(cap)
    for n in [1, 5, cap, cap + 1, cap * k, cap * k + 1, cap * k * 3 + 7, cap * k * k + 11]:
        for name, x in dists(rng, n):
            sk, si, st = model_sort(x.astype(np.int64), geo)
            ref = np.argsort(x, kind="stable")
            assert np.array_equal(si, ref), (n, name)
            for _, m in st.get("max_tile", []):
                assert m <= cap


@pytest.mark.parametrize("base", [8704, 8192])
def test_production_geometry_one_round(base):
    """Merge tiles of 8704 keys; base tiles of 8704 (key/value) or 8192
    (keys-only warp base case)."""
    geo = Geometry(8704, 32, 32, base=base)
    rng = np.random.default_rng(0)
    for name, x in dists(rng, base * 32 + 4321):
        sk, si, st = model_sort(x.astype(np.int64), geo)
        assert np.array_equal(si, np.argsort(x, kind="stable")), name
        for _, m in st.get("max_tile", []):
            assert m <= 8704


def test_base_smaller_than_merge_tile_deep():
    geo = Geometry(96, 4, 4, base=64)
    rng = np.random.default_rng(5)
    for n in [65, 256, 257, 1025, 5000]:
        for name, x in dists(rng, n):
            sk, si, st = model_sort(x.astype(np.int64), geo)
            assert np.array_equal(si, np.argsort(x, kind="stable")), (n, name)
