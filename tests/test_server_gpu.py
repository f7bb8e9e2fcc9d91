"""The sort server (gms_server_*): requests served in a concurrent mix give
the same bits as the same request sorted alone, and the latency statistics
are reported."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _alone(lib, kind, keys, vals):
    if kind == 0:
        tin = keys.clone()
        tout = torch.empty_like(keys)
        assert lib.gms_sort_i32(tin.data_ptr(), tout.data_ptr(), keys.numel(), 0, _stream()) == 0
        return tout, None
    ki, vi = keys.clone(), vals.clone()
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    assert lib.gms_sort_kv_u64_i32(ki.data_ptr(), vi.data_ptr(), ko.data_ptr(), vo.data_ptr(), keys.numel(), 0,
                                   _stream()) == 0
    return ko, vo


def test_server_mix_equals_alone(gms, oracle):
    lib = gms.load()
    rng = np.random.default_rng(11)
    srv = ctypes.c_void_p()
    assert lib.gms_server_create(8 << 30, 4, 1 << 16, 1 << 22, ctypes.byref(srv)) == 0, lib.gms_last_error()
    reqs = []
    for i in range(160):
        n = int(np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 22))))
        if rng.uniform() < 0.7:
            keys = torch.from_numpy(oracle.gen_i32(n, int(rng.integers(0, 7)), i)).cuda()
            reqs.append((0, keys, None, torch.empty_like(keys), None))
        else:
            k = oracle.gen_u64(n, i)
            k[::5] = k[0]  # ties: the payload shows stability
            keys = torch.from_numpy(k.view(np.int64)).cuda()
            vals = torch.arange(n, dtype=torch.int32, device="cuda")
            reqs.append((1, keys, vals, torch.empty_like(keys), torch.empty_like(vals)))
    torch.cuda.synchronize()  # inputs are resident before the server sees them
    ids = []
    for kind, keys, vals, ko, vo in reqs:
        rid = ctypes.c_uint64()
        rc = lib.gms_server_submit(srv, kind, keys.data_ptr(), vals.data_ptr() if vals is not None else None,
                                   ko.data_ptr(), vo.data_ptr() if vo is not None else None, keys.numel(),
                                   ctypes.byref(rid))
        assert rc == 0, lib.gms_last_error()
        ids.append(rid.value)
    lat = []
    for rid in ids:
        ms = ctypes.c_double()
        assert lib.gms_server_wait(srv, rid, ctypes.byref(ms)) == 0, lib.gms_last_error()
        lat.append(ms.value)
    assert lib.gms_server_drain(srv) == 0
    for kind, keys, vals, ko, vo in reqs:
        ak, av = _alone(lib, kind, keys, vals)
        assert torch.equal(ak, ko), "keys differ between the mix and alone"
        if kind == 1:
            assert torch.equal(av, vo), "payload differs between the mix and alone"
    # spot-check a few against the oracle as well
    for kind, keys, vals, ko, vo in reqs[:10]:
        if kind == 0:
            assert np.array_equal(ko.cpu().numpy(), oracle.sort(keys.cpu().numpy()))
    done = ctypes.c_int64()
    p50, p99, kps = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    assert lib.gms_server_stats(srv, ctypes.byref(done), ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(kps)) == 0
    assert done.value == len(reqs)
    assert 0 < p50.value <= p99.value
    assert kps.value > 0
    assert all(x > 0 for x in lat)
    assert lib.gms_server_destroy(srv) == 0


def test_server_rejects_over_budget(gms):
    lib = gms.load()
    srv = ctypes.c_void_p()
    assert lib.gms_server_create(1 << 20, 1, 1 << 10, 1 << 20, ctypes.byref(srv)) == 0
    keys = torch.zeros(1 << 20, dtype=torch.int32, device="cuda")  # needs 4 MiB staging > 1 MiB budget
    out = torch.empty_like(keys)
    rid = ctypes.c_uint64()
    assert lib.gms_server_submit(srv, 0, keys.data_ptr(), None, out.data_ptr(), None, keys.numel(),
                                 ctypes.byref(rid)) == 0
    assert lib.gms_server_wait(srv, rid.value, None) == 4  # GMS_ERR_TOO_LARGE
    assert lib.gms_server_destroy(srv) == 0
