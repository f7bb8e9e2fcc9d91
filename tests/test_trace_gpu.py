"""Per-launch trace of a host-to-host sort: kernels and both copy directions
are recorded on one device clock (gms_timing_trace)."""
import ctypes

import numpy as np
import pytest

from conftest import load_gms_module

pytestmark = pytest.mark.gpu


def test_host_sort_trace():
    torch = pytest.importorskip("torch")
    gms = load_gms_module()
    lib = gms.load()
    n = (1 << 22) + 777
    src = np.random.default_rng(5).integers(-(1 << 31), 1 << 31, n, dtype=np.int64).astype(np.int32)
    hin = torch.from_numpy(src).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
    gms.timing_collect()
    lib.gms_timing_reset()
    launches0 = lib.gms_launch_count()
    lib.gms_timing_enable(1)
    try:
        assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
    finally:
        lib.gms_timing_enable(0)
    kernels = lib.gms_launch_count() - launches0
    trace = gms.timing_trace()
    per_class = gms.timing_collect()
    assert np.array_equal(hout.numpy(), np.sort(src))
    names = [c for c, _, _ in trace]
    assert "h2d_copy" in names and "d2h_copy" in names and "base_tile_sort" in names
    # copies are traced but not counted as kernel launches
    assert len(trace) - names.count("h2d_copy") - names.count("d2h_copy") == kernels
    assert min(a for _, a, _ in trace) == 0.0
    for _, a, b in trace:
        assert 0.0 <= a <= b
    # the output leaves after the input has landed
    h2d_end = max(b for c, _, b in trace if c == "h2d_copy")
    assert max(b for c, _, b in trace if c == "d2h_copy") > h2d_end
    # the trace and the per-class totals describe the same launches
    for name, (ms, cnt) in per_class.items():
        spans = [b - a for c, a, b in trace if c == name]
        assert cnt == len(spans)
        assert ms == pytest.approx(sum(spans), rel=1e-3, abs=1e-3)
    assert gms.timing_trace() == []
