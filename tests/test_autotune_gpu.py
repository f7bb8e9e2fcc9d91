"""The autotuner (gms_autotune and the tuning table): the chosen tuning is one
of the candidates, sorts of the tuned class use it and stay bit-exact against
the oracle, an explicit gms_set_tune wins over the table, and the table
survives a save/load round trip through its JSON cache (which another GPU
model's cache cannot replace)."""
import ctypes
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DEFAULT = {"k": 32, "sample_b": 32, "bulk_copy": 1}
DEFAULT_KV = {"k": 32, "sample_b": 32, "bulk_copy": 3}  # built-in for sorts with a payload
DEFAULT_64 = DEFAULT_KV  # and for sorts of 64-bit keys


@pytest.fixture
def clean(gms):
    lib = gms.load()
    assert lib.gms_clear_tune() == 0 and lib.gms_autotune_clear() == 0
    yield lib
    assert lib.gms_clear_tune() == 0 and lib.gms_autotune_clear() == 0


def _sort(gms, a):
    t = torch.from_numpy(a).cuda()
    out = torch.empty_like(t)
    gms.sort_(t, out)
    return out.cpu().numpy()


def test_autotune_i32_class(gms, oracle, clean):
    n = (1 << 22) + 12345
    got = gms.autotune("int32", n)
    assert got["k"] in (8, 16, 32) and got["sample_b"] in (16, 32, 64) and got["bulk_copy"] in (0, 1, 2, 3)
    assert got["ms"] > 0
    chosen = {k: got[k] for k in DEFAULT}
    # same size class (floor(log2 n) = 22) uses it; others keep the defaults
    assert gms.tune_for("int32", 1 << 22) == chosen
    assert gms.tune_for("int32", (1 << 23) - 1) == chosen
    assert gms.tune_for("int32", 1 << 23) == DEFAULT
    assert gms.tune_for("uint32", 1 << 22) == DEFAULT
    assert gms.tune_for("int32", 1 << 22, kv=True) == DEFAULT_KV
    table = gms.autotune_table()
    assert len(table) == 1 and table[0]["log2n"] == 22 and table[0]["dtype"] == 0
    for dist in (0, 3, 6):
        a = oracle.gen_i32(n - 999, dist, 40 + dist)
        assert np.array_equal(_sort(gms, a), oracle.sort(a)), f"dist {dist}"
    assert gms.device_status() == 0


def test_explicit_tune_wins(gms, clean):
    gms.autotune("int32", 1 << 20)
    lib = clean
    assert lib.gms_set_tune(4, 16, 0) == 0
    assert gms.tune_for("int32", 1 << 20) == {"k": 4, "sample_b": 16, "bulk_copy": 0}
    assert lib.gms_clear_tune() == 0
    assert gms.tune_for("int32", 1 << 20) == {k: gms.autotune_table()[0][k] for k in DEFAULT}


def test_autotune_kv_f32(gms, oracle, clean):
    n = 1_500_000
    got = gms.autotune("float32", n, kv=True)
    assert gms.tune_for("float32", n, kv=True) == {k: got[k] for k in DEFAULT}
    keys = oracle.gen_f32(n, 5)
    keys[::7] = keys[3]
    vals = np.arange(n, dtype=np.int32)
    ki = torch.from_numpy(keys.view(np.int32).copy()).cuda().view(torch.float32)
    vi = torch.from_numpy(vals).cuda()
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    gms.sort_kv_(ki, vi, ko, vo)
    ok_, ov_ = oracle.sort_kv(keys, vals)
    assert np.array_equal(ko.cpu().numpy().view(np.uint32), ok_.view(np.uint32))
    assert np.array_equal(vo.cpu().numpy(), ov_)


def test_small_sizes_time_defaults_only(gms, clean):
    n = clean.gms_base_tile(4, 0) - 7  # one base tile, no merge round
    got = gms.autotune("uint64", n)
    assert {k: got[k] for k in DEFAULT} == DEFAULT


def test_cache_round_trip(gms, clean, tmp_path):
    gms.autotune("int64", 1 << 21)
    gms.autotune("uint32", 3 << 20, kv=True)
    table = gms.autotune_table()
    path = tmp_path / "tune.json"
    gms.autotune_save(path)
    doc = json.loads(path.read_text())
    assert doc["device"] == torch.cuda.get_device_name(0)
    assert len(doc["entries"]) == 2
    lib = clean
    assert lib.gms_autotune_clear() == 0
    assert gms.tune_for("int64", 1 << 21) == DEFAULT_64
    gms.autotune_load(path)
    assert sorted(map(json.dumps, gms.autotune_table())) == sorted(map(json.dumps, table))
    # another GPU model's cache is refused and leaves the table as it was
    doc["device"] = "Some Other GPU"
    doc["entries"][0]["k"] = 8
    other = tmp_path / "other.json"
    other.write_text(json.dumps(doc))
    assert lib.gms_autotune_load(str(other).encode()) == 1
    assert sorted(map(json.dumps, gms.autotune_table())) == sorted(map(json.dumps, table))
    # a malformed entry is refused as well
    bad = tmp_path / "bad.json"
    bad.write_text(path.read_text().replace('"k": ', '"k": 9'))
    assert lib.gms_autotune_load(str(bad).encode()) == 1


def test_autotune_rejects_bad_args(gms, clean):
    lib = clean
    k, b, bulk, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    args = (ctypes.byref(k), ctypes.byref(b), ctypes.byref(bulk), ctypes.byref(ms))
    assert lib.gms_autotune(6, 0, 1000, None, *args) == 1
    assert lib.gms_autotune(0, 2, 1000, None, *args) == 1
    assert lib.gms_autotune(0, 0, 0, None, *args) == 1
    assert lib.gms_autotune(0, 0, (1 << 32) + 1, None, *args) == 4
