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


@pytest.mark.parametrize("base,nt,items,int_,iitems", [(8192, 288, 31, 512, 17), (4096, 256, 17, 256, 17),
                                                        (4352, 256, 17, 256, 17)])
def test_production_geometry_one_round(base, nt, items, int_, iitems):
    """The prebuilt engines' geometries: 32-bit keys-only data rounds of
    288 x 31 (forecast tiles <= 8432 keys) with index rounds of 512 x 17;
    64-bit keys-only and key/value data and index rounds of 256 x 17 (<= 4080);
    base tiles of 8192 (32-bit keys-only warp base case), 4096 (64-bit) or
    4352 (key/value)."""
    sample = Geometry(int_ * iitems, 32, 32, nt=int_, items=iitems)
    geo = Geometry(nt * items, 32, 32, base=base, nt=nt, items=items, sample=sample)
    rng = np.random.default_rng(0)
    for name, x in dists(rng, base * 32 + 4321):
        sk, si, st = model_sort(x.astype(np.int64), geo)
        assert np.array_equal(si, np.argsort(x, kind="stable")), name
        for lev, m in st.get("max_tile", []):
            assert m <= (geo if lev == 0 else sample).tile_cap
        assert st["max_windows"] <= max(nt, int_)


@pytest.mark.parametrize("k,b", [(2, 2), (3, 2), (4, 4), (8, 2), (16, 2), (32, 2)])
def test_window_threads_fit_small_geometry(k, b):
    """Window-aligned levels on a small geometry (nt=48, items=5: forecast
    tiles of at most 160 keys, groups of 240) across fan-ins, skewed inputs
    included: every tile's levels fit the 48 threads."""
    geo = Geometry(240, k, b, base=16, nt=48, items=5)
    rng = np.random.default_rng(k * 100 + b)
    for n in [17, 300, 2000]:
        for name, x in dists(rng, n):
            sk, si, st = model_sort(x.astype(np.int64), geo)
            assert np.array_equal(si, np.argsort(x, kind="stable")), (n, name)
            assert st.get("max_windows", 0) <= 48
