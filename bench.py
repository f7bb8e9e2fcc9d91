"""Benchmark of the GB300 multiway mergesort: int32 N=2^28 keys.

One step = one full sort of N = 2^28 int32 keys drawn uniformly from
[0, 2^31-1) with a fixed seed (the reference's scale configuration), through
the C ABI (gms_sort_i32).  Each timed step sorts its own fresh copy of the
input (1 GiB per copy, far above the 129 MB L2), so no step sees a warm cache.

  value       Gkeys/s, device-resident input, the K steps timed with CUDA
              events between a barrier + synchronize on both sides
  e2e         Gkeys/s through gms_sort_host_i32 from pinned host memory:
              H2D copy + sort + D2H copy + stream wait, every step
  roofline    the dominant kernel's algorithmic bytes per launch / its mean
              launch time (CUDA events around every launch on the launching
              stream, in a second pass of the same K steps: events between
              the kernels would cancel their programmatic launch overlap in
              the timed steps), against the measured HBM copy bandwidth
  cpu_baseline std::sort (libstdc++ parallel mode, all host threads) on a
              bounded sample of the same workload (oracle, CPU only)

`--impl reference` times the CPU implementation (the oracle's std::sort with
every host thread): the reference's only CPU sort is the O(n^2) selection sort
its test driver checks small arrays with, not an implementation of the path.
Multi-GPU (torchrun): every rank sorts its own replica; no collective on the
data path ("replicas only"); value = keys of all ranks / max time over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_DEFAULT = 1 << 28
SEED = 1
PEAK_FALLBACK_GBS = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return PEAK_FALLBACK_GBS, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(dist, value, device="cuda"):
    """The job's time for a per-rank duration: its maximum over all ranks
    (replicas run concurrently, so the job ends with the slowest)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(keys_per_rank, world_size, steps, seconds):
    """Whole-job throughput in Gkeys/s: every rank's keys over the job time."""
    return keys_per_rank * world_size * steps / seconds / 1e9


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        pw = [num(r[3]) for r in rows if num(r[3]) is not None]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


def cpu_baseline(orc, n_sample, reps=3, threads=None):
    """std::sort, libstdc++ parallel mode, every host thread (or `threads`), on
    n_sample keys."""
    import numpy as np

    threads = threads or os.cpu_count() or 1
    a = orc.gen_i32(n_sample, 0, SEED)
    best = None
    for _ in range(reps):
        b = a.copy()
        t0 = time.perf_counter()
        used = orc.lib.gmo_par_sort_i32(ctypes.c_void_p(b.ctypes.data), b.size, threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    assert np.all(b[1:] >= b[:-1])
    return {"value": round(n_sample / best / 1e9, 4), "unit": "Gkeys/s", "cores": int(used),
            "kind": "port", "sample": f"{n_sample} int32 keys of the same distribution, std::sort "
            f"(__gnu_parallel) on {int(used)} threads, best of {reps}"}


def log_uniform_lengths(rng, lo, hi, total_cap=None, count=None):
    """Segment lengths log-uniform in [lo, hi] until `count` or `total_cap`."""
    import numpy as np

    out = []
    tot = 0
    while True:
        if count is not None and len(out) >= count:
            break
        v = int(np.exp(rng.uniform(np.log(lo), np.log(hi + 1))))
        v = min(max(v, lo), hi)
        if total_cap is not None and tot + v > total_cap:
            break
        out.append(v)
        tot += v
    return np.array(out, dtype=np.int64)


DIST_NAMES = ["uniform", "sorted", "reverse", "all_equal", "16_values", "zipf_1.2"]


def _sort_time(lib, fn, srcs, outs, n, reps, stream):
    """Median CUDA-event time (ms) of one sort call on a fresh device copy of
    the inputs per repetition (the copy is outside the events)."""
    import torch

    work = [t.clone() for t in srcs]
    sp = ctypes.c_void_p(stream.cuda_stream)
    times = []
    with torch.cuda.stream(stream):
        for r in range(reps + 1):  # the first run warms up
            for w, t in zip(work, srcs):
                w.copy_(t)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if len(srcs) == 1:
                rc = fn(work[0].data_ptr(), outs[0].data_ptr(), n, 0, sp)
            else:
                rc = fn(work[0].data_ptr(), work[1].data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(), n, 0, sp)
            e1.record(stream)
            assert rc == 0, lib.gms_last_error()
            stream.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def config_sweep(lib, orc, peak, reps=5):
    """The other sizes, distributions and key/value layouts of the workload
    set: int32 2^24 uniform; int32 2^28 in the five non-uniform distributions;
    2^27 uint64 keys + int32 payload and 2^27 float32 keys + int32 payload.
    Each entry: Gkeys/s (median of `reps`), the fraction of the whole-sort
    HBM roofline 2*N*bytes_per_element*(1+rounds) at the measured peak, and a
    bit-exact check against a (stable) torch.sort of the same data."""
    import numpy as np
    import torch

    stream = torch.cuda.Stream()
    out = {}

    def entry(n, ms, elt_bytes, dtype_code, kv, ok):
        passes = 1 + int(lib.gms_rounds(dtype_code, kv, n))
        gbs = 2 * n * elt_bytes * passes / (ms * 1e-3) / 1e9
        return {"n": n, "gkeys_s": round(n / ms / 1e6, 3), "ms": round(ms, 4), "passes": passes,
                "sort_roofline_frac": round(gbs / peak, 4), "bit_exact": ok}

    # int32, 2^24 uniform and 2^28 in each non-uniform distribution
    for n, dists in ((1 << 24, [0]), (1 << 28, [1, 2, 3, 4, 5])):
        for d in dists:
            src = torch.from_numpy(orc.gen_i32(n, d, SEED)).cuda()
            dst = torch.empty_like(src)
            ms = _sort_time(lib, lib.gms_sort_i32, [src], [dst], n, reps, stream)
            ok = bool(torch.equal(dst, torch.sort(src)[0]))
            out[f"int32_{DIST_NAMES[d]}_2p{n.bit_length() - 1}"] = entry(n, ms, 4, 0, 0, ok)
            del src, dst
            torch.cuda.empty_cache()
    # key/value: 2^27 uint64 + int32 index, 2^27 float32 + int32 index
    n = 1 << 27
    k64 = orc.gen_u64(n, SEED)
    kf = orc.gen_f32(n, SEED)
    for name, keys, fn, code, kb in (("uint64_kv_i32_2p27", k64.view(np.int64), lib.gms_sort_kv_u64_i32, 4, 8),
                                     ("float32_kv_i32_2p27", kf.view(np.int32), lib.gms_sort_kv_f32_i32, 2, 4)):
        kt = torch.from_numpy(keys).cuda()
        vt = torch.arange(n, dtype=torch.int32, device="cuda")
        ko, vo = torch.empty_like(kt), torch.empty_like(vt)
        ms = _sort_time(lib, fn, [kt, vt], [ko, vo], n, reps, stream)
        # expected order from a stable torch.sort of order-preserving signed images of the keys
        if kb == 8:
            img = kt ^ torch.tensor(-(1 << 63), dtype=torch.int64, device="cuda")
        else:
            img = kt ^ ((kt >> 31) & 0x7FFFFFFF)
        _, idx = torch.sort(img, stable=True)
        ok = bool(torch.equal(vo, idx.to(torch.int32)) and torch.equal(ko, kt[idx]))
        del img, idx
        out[name] = entry(n, ms, kb + 4, code, 1, ok)
        del kt, vt, ko, vo
        torch.cuda.empty_cache()
    return out


def dropin_bench(lib, orc, n, iters=5):
    """The reference's own call, multimergesort<int, cmp<int>> from the
    header-only drop-in, through the testMM-compatible driver (its input:
    srand(0), rand()%1024 per key), against gms_sort_i32 on the same keys
    (the reference generator reproduced by the oracle)."""
    import torch

    exe = os.path.join(ROOT, "gpu-mms_gb300", "testmm")
    if not os.path.exists(exe):
        return {"unavailable": "testmm not built"}
    r = subprocess.run([exe, str(n), str(iters)], capture_output=True, text=True, timeout=900)
    lines = r.stdout.strip().splitlines()
    if r.returncode != 0 or len(lines) < 2:
        return {"unavailable": f"testmm exited {r.returncode}: {r.stderr.strip()[:200]}"}
    avg, lo, hi = (float(x) for x in lines[0].split())
    src = torch.from_numpy(orc.ref_random_list(n, 0)).cuda()
    dst = torch.empty_like(src)
    ms_capi = _sort_time(lib, lib.gms_sort_i32, [src], [dst], n, iters, torch.cuda.Stream())
    return {"workload": f"testmm {n} {iters}: multimergesort<int, cmp<int>>, keys rand()%1024 (srand(0))",
            "dropin_ms_min": round(lo, 4), "dropin_ms_avg": round(avg, 4), "sorted": lines[1] == "SORTED!",
            "c_abi_ms": round(ms_capi, 4), "dropin_gkeys_s": round(n / lo / 1e6, 3),
            "dropin_vs_c_abi": round(ms_capi / lo, 3)}


def library_baselines(n, reps=5):
    """thrust::sort on the same kind of input: CUB radix sort (keys only) and
    CUB merge sort (user comparator), from the in-tree thrust_baseline program."""
    exe = os.path.join(ROOT, "gpu-mms_gb300", "thrust_baseline")
    if not os.path.exists(exe):
        return {"unavailable": "thrust_baseline not built"}
    r = subprocess.run([exe, str(n), str(reps)], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"unavailable": f"thrust_baseline exited {r.returncode}: {r.stderr.strip()[:200]}"}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    d["what"] = "thrust::sort int32 uniform: radix = keys-only (CUB radix sort), merge = user comparator (CUB merge sort)"
    r = subprocess.run([exe, str(1 << 27), str(reps), "kv64"], capture_output=True, text=True, timeout=600)
    if r.returncode == 0:
        d["kv64"] = json.loads(r.stdout.strip().splitlines()[-1])
        d["kv64"]["what"] = "thrust::stable_sort_by_key, 2^27 uint64 keys + int32 payload: radix / user comparator"
    return d


def batched_bench(lib, orc, total_keys, nseg=None, seed=7):
    """Config 4: many int32 arrays, lengths log-uniform in [32, 2^20]; one
    batched (segmented) sort vs its CUDA-graph replay vs one plain call per
    array, all device-resident, bit-exact per array."""
    import numpy as np
    import torch

    rng = np.random.default_rng(seed)
    lengths = log_uniform_lengths(rng, 32, 1 << 20, total_cap=total_keys, count=nseg)
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    n = int(off[-1])
    if n <= (1 << 30):
        keys = torch.from_numpy(orc.gen_i32(n, 0, seed)).cuda()
    else:
        # billions of keys: drawn on the device (uniform in [0, 2^31-1), seeded)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        keys = torch.randint(0, (1 << 31) - 1, (n,), dtype=torch.int32, device="cuda", generator=gen)
    toff = torch.from_numpy(off).cuda()
    out = torch.empty_like(keys)
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)

    def ev_time(fn, reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s):
            fn()  # warm-up
            s.synchronize()
            e0.record(s)
            for _ in range(reps):
                fn()
            e1.record(s)
            s.synchronize()
        return e0.elapsed_time(e1) / reps

    def batched():
        assert lib.gms_segmented_sort_i32(keys.data_ptr(), out.data_ptr(), n, toff.data_ptr(), len(lengths), sp) == 0

    t_batched = ev_time(batched, 3)
    batched_out = out.clone()
    g = ctypes.c_void_p()
    with torch.cuda.stream(s):
        assert lib.gms_graph_create_segmented_i32(keys.data_ptr(), out.data_ptr(), n, toff.data_ptr(), len(lengths),
                                                  sp, ctypes.byref(g)) == 0
    t_graph = ev_time(lambda: lib.gms_graph_launch(g, sp), 3)
    lib.gms_graph_destroy(g)
    # plain: one gms_sort_i32 call per array (input copies made beforehand)
    work = keys.clone()
    plain_out = torch.empty_like(keys)

    def plain():
        for i in range(len(lengths)):
            a = int(off[i])
            m = int(lengths[i])
            assert lib.gms_sort_i32(work.data_ptr() + 4 * a, plain_out.data_ptr() + 4 * a, m, 0, sp) == 0

    with torch.cuda.stream(s):
        work.copy_(keys)
    t_plain = ev_time(lambda: (work.copy_(keys), plain()), 1) - ev_time(lambda: work.copy_(keys), 3)
    same = bool(torch.equal(plain_out, batched_out))
    return {
        "workload": f"{len(lengths)} int32 arrays, lengths log-uniform in [32, 2^20], {n} keys in all, uniform keys"
                    + (f" (the first arrays that fit {total_keys} keys)" if nseg is None else ""),
        "keys": n, "arrays": int(len(lengths)),
        "batched_gkeys_s": round(n / t_batched / 1e6, 3), "batched_ms": round(t_batched, 3),
        "graph_gkeys_s": round(n / t_graph / 1e6, 3), "graph_ms": round(t_graph, 3),
        "plain_calls_gkeys_s": round(n / t_plain / 1e6, 3), "plain_calls_ms": round(t_plain, 3),
        "speedup_vs_plain": round(t_plain / min(t_batched, t_graph), 2),
        "bit_exact_vs_plain": same,
    }


def serving_bench(lib, orc, seconds, rate=2000.0, lo=1 << 10, hi=1 << 26, budget=64 << 30, seed=9):
    """Config 5: Poisson arrivals, sizes log-uniform in [lo, hi], 70% int32 /
    30% uint64 key + int32 payload, device-resident inputs, admission by a
    device-memory budget, continuous batching; p50/p99 latency and keys/s vs
    the same requests sorted by serial plain calls."""
    import numpy as np
    import torch

    rng = np.random.default_rng(seed)
    count = None
    if rate <= 0:
        # capacity run: as many requests as 2000 req/s would bring, all at t=0
        count = int((20000 if hi <= (1 << 16) else 2000) * seconds)
    pool32 = torch.from_numpy(orc.gen_i32(1 << 28, 0, seed)).cuda()
    pool64 = torch.from_numpy(orc.gen_u64(1 << 27, seed).view(np.int64)).cuda()
    poolv = torch.arange(1 << 27, dtype=torch.int32, device="cuda")
    t = 0.0
    reqs = []
    while (t < seconds) if count is None else (len(reqs) < count):
        t = t + rng.exponential(1.0 / rate) if count is None else 0.0
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi + 1))))
        n = min(max(n, lo), hi)
        kind = 0 if rng.uniform() < 0.7 else 1
        cap = (1 << 28) if kind == 0 else (1 << 27)
        n = min(n, cap)
        o = int(rng.integers(0, cap - n + 1))
        reqs.append((t, kind, n, o))
    torch.cuda.synchronize()
    # outputs come from preallocated rings: no allocation inside the arrival loop
    ring32 = torch.empty(1 << 30, dtype=torch.int32, device="cuda")
    ring64 = torch.empty(1 << 29, dtype=torch.int64, device="cuda")
    ringv = torch.empty(1 << 29, dtype=torch.int32, device="cuda")
    pos = [0, 0]
    srv = ctypes.c_void_p()
    assert lib.gms_server_create(budget, 8, 1 << 16, hi, ctypes.byref(srv)) == 0, lib.gms_last_error()
    ids = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for (ta, kind, n, o) in reqs:
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        cap = ring32.numel() if kind == 0 else ring64.numel()
        if pos[kind] + n > cap:
            pos[kind] = 0
        r0 = pos[kind]
        pos[kind] += (n + 63) & ~63
        if kind == 0:
            kin, vin = pool32.data_ptr() + 4 * o, None
            kout, vout = ring32.data_ptr() + 4 * r0, None
        else:
            kin, vin = pool64.data_ptr() + 8 * o, poolv.data_ptr() + 4 * o
            kout, vout = ring64.data_ptr() + 8 * r0, ringv.data_ptr() + 4 * r0
        rid = ctypes.c_uint64()
        assert lib.gms_server_submit(srv, kind, kin, vin, kout, vout, n, ctypes.byref(rid)) == 0
        ids.append(rid.value)
    assert lib.gms_server_drain(srv) == 0, lib.gms_last_error()
    wall = time.perf_counter() - t0
    done = ctypes.c_int64()
    p50, p99, kps = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib.gms_server_stats(srv, ctypes.byref(done), ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(kps))
    for rid in ids:
        lib.gms_server_wait(srv, rid, None)
    lib.gms_server_destroy(srv)
    del ring32, ring64, ringv
    keys_total = sum(r[2] for r in reqs)
    # the same requests, serially, one plain call each (device-resident)
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    tmp32 = torch.empty(hi, dtype=torch.int32, device="cuda")
    out32 = torch.empty_like(tmp32)
    tmp64 = torch.empty(min(hi, 1 << 27), dtype=torch.int64, device="cuda")
    out64 = torch.empty_like(tmp64)
    tmpv = torch.empty(min(hi, 1 << 27), dtype=torch.int32, device="cuda")
    outv = torch.empty_like(tmpv)
    torch.cuda.synchronize()
    # one event after every request: the serial time each request takes
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(reqs) + 1)]
    ts = time.perf_counter()
    with torch.cuda.stream(s):
        evs[0].record(s)
        for i, (_, kind, n, o) in enumerate(reqs):
            if kind == 0:
                tmp32[:n].copy_(pool32[o:o + n])
                assert lib.gms_sort_i32(tmp32.data_ptr(), out32.data_ptr(), n, 0, sp) == 0
            else:
                tmp64[:n].copy_(pool64[o:o + n])
                tmpv[:n].copy_(poolv[o:o + n])
                assert lib.gms_sort_kv_u64_i32(tmp64.data_ptr(), tmpv.data_ptr(), out64.data_ptr(), outv.data_ptr(),
                                               n, 0, sp) == 0
            evs[i + 1].record(s)
        s.synchronize()
    serial = time.perf_counter() - ts
    # How much of the serial time the requests of at least 2^20 keys take:
    # one plain call already sorts those with full grids, so batching can only
    # remove the time of the smaller ones (the gain beyond that comes from
    # running requests side by side on several streams)
    per_req = [evs[i].elapsed_time(evs[i + 1]) * 1e-3 for i in range(len(reqs))]
    big_s = sum(t for t, r in zip(per_req, reqs) if r[2] >= (1 << 20))
    big_keys = sum(r[2] for r in reqs if r[2] >= (1 << 20))
    return {
        "workload": (f"Poisson {rate:.0f} req/s for {seconds} s" if count is None else
                     f"{count} requests all arriving at once (capacity)") +
                    f", sizes log-uniform [{lo}, {hi}], 70% int32 / 30% uint64+int32, {budget >> 30} GB budget, "
                    "8 streams, batching <= 65536 keys",
        "requests": len(reqs), "completed": int(done.value), "keys": keys_total,
        "p50_ms": round(p50.value, 3), "p99_ms": round(p99.value, 3),
        "served_gkeys_s": round(kps.value / 1e9, 3), "wall_s": round(wall, 3),
        "serial_plain_gkeys_s": round(keys_total / serial / 1e9, 3), "serial_plain_s": round(serial, 3),
        "serial_keys_share_ge_2p20": round(big_keys / max(keys_total, 1), 4),
        "serial_time_share_ge_2p20": round(big_s / max(sum(per_req), 1e-12), 4),
        **({"speedup_vs_serial": round(serial / max(wall, 1e-9), 2),
            "if_small_free_vs_serial": round(sum(per_req) / big_s, 2) if big_s > 0 else None}
           if count is not None else
           {"kept_up": bool(wall <= seconds * 1.05 + 0.05),
            "offered_gkeys_s": round(keys_total / seconds / 1e9, 3)}),
    }


def host_trace(lib, gms, orc, n, warmup=3, trace_out=None):
    """Timeline of one synchronous host-to-host sort (gms_sort_host_i32):
    every kernel and every input / output copy bracketed by CUDA events on its
    own stream.  The events add a few microseconds per launch, so the plain
    (untraced) call time is reported beside the traced one."""
    import numpy as np
    import torch

    src = orc.gen_i32(n, 0, SEED)
    hin = torch.from_numpy(src).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(max(warmup, 3)):  # also the first device accesses to fresh pinned pages
        assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
    plain = []
    for _ in range(5):
        t0 = time.perf_counter()
        assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
        plain.append(time.perf_counter() - t0)
    gms.timing_collect()  # nothing pending from earlier calls
    lib.gms_timing_reset()
    lib.gms_timing_enable(1)
    assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
    lib.gms_timing_enable(0)
    trace = gms.timing_trace()
    per_class = gms.timing_collect()
    h = hout.numpy()
    # sorted, and the same multiset by sum and xor (a cheap check at full size)
    ok = bool(np.all(h[1:] >= h[:-1]) and h.astype(np.int64).sum() == src.astype(np.int64).sum()
              and np.bitwise_xor.reduce(h) == np.bitwise_xor.reduce(src))
    copies = ("h2d_copy", "d2h_copy")
    kern = [(c, a, b) for c, a, b in trace if c not in copies]
    h2d = [(a, b) for c, a, b in trace if c == "h2d_copy"]
    d2h = [(a, b) for c, a, b in trace if c == "d2h_copy"]
    h2d_end = max(b for _, b in h2d)
    d2h_start = min(a for a, _ in d2h)
    d2h_end = max(b for _, b in d2h)
    h2d_busy = sum(b - a for a, b in h2d)
    d2h_busy = sum(b - a for a, b in d2h)
    # the host link: each direction alone, and both at once on two streams
    dev = [torch.empty_like(hin, device="cuda") for _ in range(2)]
    side = [torch.cuda.Stream(), torch.cuda.Stream()]

    def copy_ms(h2d, d2h_too, reps=3):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if h2d:
                with torch.cuda.stream(side[0]):
                    dev[0].copy_(hin, non_blocking=True)
            if d2h_too:
                with torch.cuda.stream(side[1]):
                    hout.copy_(dev[1], non_blocking=True)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return best

    copy_ms(True, True, 1)
    link = {"h2d_gbs": round(n * 4 / copy_ms(True, False) / 1e9, 1),
            "d2h_gbs": round(n * 4 / copy_ms(False, True) / 1e9, 1),
            "both_directions_gbs": round(2 * n * 4 / copy_ms(True, True) / 1e9, 1)}
    del dev
    if trace_out:
        with open(trace_out, "w") as f:
            f.write("class,start_ms,end_ms\n")
            for c, a, b in trace:
                f.write(f"{c},{a:.4f},{b:.4f}\n")
    return {
        "n": n,
        "correct": ok,
        "plain_ms_median": round(statistics.median(plain) * 1e3, 3),
        "traced_ms": round(d2h_end, 3),
        "entries": len(trace),
        "input_landed_ms": round(h2d_end, 3),
        "first_output_copy_ms": round(d2h_start, 3),
        "kernels_end_ms": round(max(b for _, _, b in kern), 3),
        "output_landed_ms": round(d2h_end, 3),
        "h2d_gbs": round(n * 4 / (h2d_busy * 1e-3) / 1e9, 1),
        "d2h_gbs": round(n * 4 / (d2h_busy * 1e-3) / 1e9, 1),
        "kernel_busy_ms": round(sum(b - a for _, a, b in kern), 3),
        "per_class_ms": {k: round(v[0], 3) for k, v in per_class.items() if v[1]},
        "per_class_launches": {k: int(v[1]) for k, v in per_class.items() if v[1]},
        "link": link,
    }


def summarize(d):
    """Compact per-configuration results: [Gkeys/s, fraction of the whole-sort
    HBM roofline, bit-exact] per plain / key-value configuration, and the
    headline figure of each other section."""
    out = {}
    for k, v in d.get("configs", {}).items():
        out[k] = [v["gkeys_s"], v["sort_roofline_frac"], v["bit_exact"]]
    dr = d.get("dropin", {})
    if "dropin_gkeys_s" in dr:
        out["dropin_int_2p28"] = {"gkeys_s": dr["dropin_gkeys_s"], "vs_c_abi": dr["dropin_vs_c_abi"],
                                  "sorted": dr["sorted"]}
    lb = d.get("library_baselines", {})
    if "radix_gkeys_s" in lb:
        out["cub_radix_merge_gkeys_s"] = [lb["radix_gkeys_s"], lb["merge_gkeys_s"]]
    b = d.get("batched", {})
    if "batched_gkeys_s" in b:
        out["batched_c4"] = {"arrays": b["arrays"], "keys": b["keys"], "gkeys_s": b["batched_gkeys_s"],
                             "graph_gkeys_s": b["graph_gkeys_s"], "vs_plain": b["speedup_vs_plain"],
                             "exact": b["bit_exact_vs_plain"]}
    for k in ("serving", "serving_capacity", "serving_small", "serving_small_capacity"):
        v = d.get(k)
        if v:
            e = {"p50_ms": v["p50_ms"], "p99_ms": v["p99_ms"], "gkeys_s": v["served_gkeys_s"]}
            if "speedup_vs_serial" in v:
                e["vs_serial"] = v["speedup_vs_serial"]
                if v.get("if_small_free_vs_serial"):
                    e["if_small_free_vs_serial"] = v["if_small_free_vs_serial"]
            else:
                e["kept_up"] = v["kept_up"]
            out[k] = e
    return out


def profile_run(lib, orc, args):
    """Warm-up + 1 calls of one workload and nothing else, for ncu captures of
    the kernels it launches: int32 / u64 keys-only sorts, u64 / float32 keys
    with an int32 payload, a batched int32 sort (arrays log-uniform in [32,
    2^20] up to --n keys), or co-ranks of 32 runs at 8192 ranks."""
    import numpy as np
    import torch

    n = args.n
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if args.bulk_copy is not None:
        assert lib.gms_set_tune(32, 32, args.bulk_copy) == 0, lib.gms_last_error()
    calls = args.warmup + 1
    if args.what in ("int32", "u64"):
        src = torch.from_numpy(orc.gen_i32(n, 0, SEED) if args.what == "int32"
                               else orc.gen_u64(n, SEED).view(np.int64)).cuda()
        fn = lib.gms_sort_i32 if args.what == "int32" else lib.gms_sort_u64
        tin, tout = torch.empty_like(src), torch.empty_like(src)
        for _ in range(calls):
            tin.copy_(src)
            assert fn(tin.data_ptr(), tout.data_ptr(), n, 0, sp) == 0, lib.gms_last_error()
    elif args.what in ("kv_u64", "kv_f32"):
        keys = orc.gen_u64(n, SEED).view(np.int64) if args.what == "kv_u64" else orc.gen_f32(n, SEED).view(np.int32)
        src = torch.from_numpy(keys).cuda()
        vals = torch.arange(n, dtype=torch.int32, device="cuda")
        fn = lib.gms_sort_kv_u64_i32 if args.what == "kv_u64" else lib.gms_sort_kv_f32_i32
        ki, vi = torch.empty_like(src), torch.empty_like(vals)
        ko, vo = torch.empty_like(src), torch.empty_like(vals)
        for _ in range(calls):
            ki.copy_(src)
            vi.copy_(vals)
            assert fn(ki.data_ptr(), vi.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, 0, sp) == 0, lib.gms_last_error()
    elif args.what == "batched":
        rng = np.random.default_rng(7)
        lengths = log_uniform_lengths(rng, 32, 1 << 20, total_cap=n)
        off = np.zeros(len(lengths) + 1, dtype=np.int64)
        np.cumsum(lengths, out=off[1:])
        n = int(off[-1])
        src = torch.from_numpy(orc.gen_i32(n, 0, SEED)).cuda()
        toff = torch.from_numpy(off).cuda()
        out = torch.empty_like(src)
        for _ in range(calls):
            assert lib.gms_segmented_sort_i32(src.data_ptr(), out.data_ptr(), n, toff.data_ptr(), len(lengths),
                                              sp) == 0, lib.gms_last_error()
    else:
        # co-ranks: 32 sorted runs of n/32 keys, 8192 equal-share ranks
        size = max(1, n // 32)
        runs = np.sort(orc.gen_i32(size * 32, 0, SEED).reshape(32, size), axis=1).reshape(-1)
        task = torch.from_numpy(runs).cuda()
        ranks = torch.linspace(0, size * 32, 8192, dtype=torch.float64).to(torch.int64).cuda()
        outc = torch.empty((8192, 32), dtype=torch.int64, device="cuda")
        for _ in range(calls):
            assert lib.gms_find_partitions_i32(task.data_ptr(), size, 32, size * 32, ranks.data_ptr(), 8192,
                                               outc.data_ptr(), sp) == 0, lib.gms_last_error()
    torch.cuda.synchronize()
    print(json.dumps({"mode": "profile", "what": args.what, "n": n, "calls": calls}), flush=True)
    return 0


def run_reference(args):
    """CPU arm: the oracle's std::sort with every host thread."""
    import numpy as np
    from conftest import Oracle

    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    orc = Oracle()
    n = args.n
    threads = os.cpu_count() or 1
    src = orc.gen_i32(n, 0, SEED)
    # one untimed probe decides whether a step can take the full workload
    probe = src.copy()
    t0 = time.perf_counter()
    orc.lib.gmo_par_sort_i32(ctypes.c_void_p(probe.ctypes.data), probe.size, threads)
    per_full = time.perf_counter() - t0
    budget_s = 150.0
    sample = n if per_full * (args.steps + args.warmup) <= budget_s else max(1 << 20, n >> 2)
    work = src[:sample]
    times = []
    for i in range(args.warmup + args.steps):
        b = work.copy()
        t0 = time.perf_counter()
        used = orc.lib.gmo_par_sort_i32(ctypes.c_void_p(b.ctypes.data), b.size, threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    assert np.all(b[1:] >= b[:-1])
    tot = sum(times)
    value = sample * len(times) / tot / 1e9
    line = {
        "metric": "Gkeys/s int32 N=2^28", "value": round(value, 4), "unit": "Gkeys/s", "impl": "reference",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot / len(times) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: uniform int32 in [0, 2^31-1), mt19937_64 seed 1",
        "config": {"workload": f"int32 N={n} uniform sort on the host CPU", "n": n, "sample": sample},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gkeys/s", "cores": int(used), "kind": "port",
                         "sample": f"{sample} keys per step, std::sort (__gnu_parallel) on {int(used)} threads; "
                                   "the reference's only CPU sort is its test driver's O(n^2) selection sort, "
                                   "so this is the oracle's std::sort"},
        "e2e": {"value": round(value, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch
    from conftest import Oracle, load_gms_module

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    gms = load_gms_module()
    gms.build()
    lib = gms.load()
    orc = Oracle()
    n = args.n
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    src_h = orc.gen_i32(n, 0, SEED + rank)
    src = torch.from_numpy(src_h).cuda()
    ncopies = max(args.steps, args.warmup)
    inputs = [torch.empty_like(src) for _ in range(ncopies)]
    out = torch.empty_like(src)
    autotuned = gms.autotune("int32", n, stream=stream) if args.autotune else None
    tune = gms.tune_for("int32", n)
    assert lib.gms_reserve(0, 0, n, sp) == 0

    def refill(k):
        for t in inputs[:k]:
            t.copy_(src)
        torch.cuda.synchronize()

    def sort_one(t):
        rc = lib.gms_sort_i32(t.data_ptr(), out.data_ptr(), n, 0, sp)
        if rc != 0:
            raise RuntimeError(lib.gms_last_error().decode())

    # warm-up
    refill(args.warmup)
    for i in range(args.warmup):
        sort_one(inputs[i])
    torch.cuda.synchronize()
    # correctness of the last warm-up result (full-size, bit-exact vs torch.sort)
    ok = bool(torch.equal(out, torch.sort(src)[0]))
    refill(args.steps)

    # ---- timed region ----
    # Per-launch events would sit between the sort's kernels and cancel their
    # programmatic launch overlap, so the timed steps run without them and a
    # second pass of the same steps (below) gives the per-kernel split.
    launches0 = lib.gms_launch_count()
    gpu_index = local
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        try:
            gpu_index = int(vis.split(",")[local])
        except ValueError:
            pass
    with ClockSampler(gpu_index) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            sort_one(inputs[i])
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    launches = lib.gms_launch_count() - launches0
    # the last timed sort's output, bit-exact against torch.sort
    ok_timed = bool(torch.equal(out, torch.sort(src)[0]))
    ms_total = e0.elapsed_time(e1)
    # per-kernel split: the same steps again, each launch bracketed by events
    refill(args.steps)
    lib.gms_timing_reset()
    lib.gms_timing_enable(1)
    for i in range(args.steps):
        sort_one(inputs[i])
    torch.cuda.synchronize()
    lib.gms_timing_enable(0)
    per_kernel = gms.timing_collect()
    ms_total = max_over_ranks(dist, ms_total)
    ms_step = ms_total / args.steps
    value = job_rate(n, ws, args.steps, ms_total * 1e-3)

    # ---- end to end through the C ABI with host buffers ----
    hin = torch.from_numpy(src_h).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    for _ in range(3):  # untimed: the first device accesses to fresh pinned pages are slow
        assert lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp) == 0
    # five timed batches of e2e_steps calls; the median counts (the host link
    # is shared with other tenants' jobs, so a batch can be slowed from outside)
    e2e_steps = min(args.steps, 5)
    e2e_batches = 5
    sync_reps = []
    for _ in range(e2e_batches):
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            rc = lib.gms_sort_host_i32(hin.data_ptr(), hout.data_ptr(), n, sp)
            assert rc == 0, lib.gms_last_error()
        torch.cuda.synchronize()
        sync_reps.append((time.perf_counter() - t0) / e2e_steps)
    e2e_s = max_over_ranks(dist, statistics.median(sync_reps))
    e2e_ok = bool(np.array_equal(hout.numpy(), out.cpu().numpy()))
    # pipelined: the same host-to-host sorts with calls in flight (the input
    # copy of step i+1 and the output copy of step i-1 overlap the sort of
    # step i); each batch starts and ends empty, so its first input copy and
    # last output copy overlap nothing
    pipe_steps = max(e2e_steps, 10)
    houts = [hout, torch.empty_like(hin).pin_memory()]
    for i in range(6):  # untimed: first device accesses to each pinned buffer and buffer set
        assert lib.gms_sort_host_i32_async(hin.data_ptr(), houts[i % 2].data_ptr(), n, sp) == 0
    assert lib.gms_host_sync(sp) == 0
    reps = []
    for _ in range(e2e_batches):  # timed batches of pipe_steps calls; the median counts
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(pipe_steps):
            rc = lib.gms_sort_host_i32_async(hin.data_ptr(), houts[i % 2].data_ptr(), n, sp)
            assert rc == 0, lib.gms_last_error()
        assert lib.gms_host_sync(sp) == 0
        reps.append((time.perf_counter() - t0) / pipe_steps)
    pipe_s = max_over_ranks(dist, statistics.median(reps))
    pipe_ok = all(bool(np.array_equal(h.numpy(), houts[0].numpy())) for h in houts[1:]) and e2e_ok

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel ----
    peak, peak_kind = peaks()
    rounds = int(lib.gms_rounds(0, 0, n))
    passes = 1 + rounds
    bytes_per_pass = 2 * n * 4
    dom = max(per_kernel.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_launches) = dom
    dom_avg_ms = dom_ms / max(dom_launches, 1)
    achieved = bytes_per_pass / (dom_avg_ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(dom_name)
    sort_bytes = bytes_per_pass * passes
    line = {
        "metric": "Gkeys/s int32 N=2^28",
        "value": round(value, 3),
        "unit": "Gkeys/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic: uniform int32 in [0, 2^31-1), mt19937_64 seed 1 (+rank)",
        "config": {
            "workload": f"multimergesort int32 N={n} uniform, one full sort per step",
            "n": n, "rounds": rounds, "passes": passes, "base_tile": int(lib.gms_base_tile(0, 0)), "k": tune["k"],
            "sample_block": tune["sample_b"], "bulk_copy": tune["bulk_copy"],
            "tuning": "autotuned before warm-up" if autotuned else "defaults",
            "parallelism": "replicas" if ws > 1 else "single",
            "l2": "each step sorts its own 1 GiB input copy (> 129 MB L2)",
            "correct": ok and ok_timed and e2e_ok,
            "correct_checked": "last warm-up output, last timed output and the end-to-end output, "
                               "bit-exact against torch.sort",
        },
        "roofline": {
            "bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
            "bytes_per_launch": bytes_per_pass, "mean_launch_ms": round(dom_avg_ms, 4),
            "traffic": traffic,
            "sort_frac": round(sort_bytes / (ms_step * 1e-3) / 1e9 / peak, 4),
            "launch_times": "CUDA events around each launch, second pass of the same steps",
        },
        "per_kernel_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in per_kernel.items() if v[1]},
        "e2e": {"value": round(job_rate(n, ws, 1, e2e_s), 3), "unit": "Gkeys/s", "h2d_bytes_per_step": n * 4,
                "d2h_bytes_per_step": n * 4, "ms_per_step": round(e2e_s * 1e3, 3),
                "batches_ms_per_step": [round(x * 1e3, 3) for x in sync_reps],
                "api": "gms_sort_host_i32 (synchronous, one call per step)"},
        "e2e_pipelined": {"value": round(job_rate(n, ws, 1, pipe_s), 3), "unit": "Gkeys/s",
                          "h2d_bytes_per_step": n * 4,
                          "d2h_bytes_per_step": n * 4, "ms_per_step": round(pipe_s * 1e3, 3), "correct": pipe_ok,
                          "batches_ms_per_step": [round(x * 1e3, 3) for x in reps],
                          "calls_per_batch": pipe_steps,
                          "api": "gms_sort_host_i32_async, calls in flight, gms_host_sync at the end of a batch"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(orc, min(n, 1 << 26))
    details = {}
    if not args.no_cpu:
        details["cpu_baseline_1thread"] = cpu_baseline(orc, min(n, 1 << 24), reps=1, threads=1)
    if not args.no_extra:
        del inputs
        torch.cuda.empty_cache()
        details["configs"] = config_sweep(lib, orc, peak)
        details["dropin"] = dropin_bench(lib, orc, n)
        details["library_baselines"] = library_baselines(n)
        # the batched and serving configurations as stated: 50,000 arrays;
        # Poisson arrivals for 60 s
        details["batched"] = batched_bench(lib, orc, total_keys=None, nseg=50000)
        torch.cuda.empty_cache()
        details["serving"] = serving_bench(lib, orc, seconds=60.0)
        details["serving_capacity"] = serving_bench(lib, orc, seconds=2.0, rate=0)
        details["serving_small"] = serving_bench(lib, orc, seconds=1.0, rate=20000.0, hi=1 << 16)
        details["serving_small_capacity"] = serving_bench(lib, orc, seconds=1.0, rate=0, hi=1 << 16)
    # every section in full on a line of its own, then the one JSON line with
    # a compact summary at its end (a reader of the output's tail sees it)
    if details:
        print("details " + json.dumps(details), flush=True)
        line["summary"] = summarize(details)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--keys", dest="n", type=int, default=N_DEFAULT,
                    help="keys per sort (--keys also works under torchrun, whose own options --n would prefix)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--autotune", action="store_true", help="run gms_autotune for the workload before warm-up")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and serving sections")
    ap.add_argument("--mode", default="sort", choices=["sort", "batched", "serve", "profile", "trace"],
                    help="sort: the headline line; batched / serve: the full-size config 4 / config 5 runs; "
                         "profile: warm-up sorts plus one sort of --n keys and nothing else (for ncu); "
                         "trace: the timeline of one synchronous host-to-host sort of --n keys")
    ap.add_argument("--trace-out", default=None, help="trace mode: also write every launch and copy as CSV here")
    ap.add_argument("--what", default="int32", choices=["int32", "u64", "kv_u64", "kv_f32", "batched", "corank"],
                    help="profile mode: the workload (each runs warm-up + 1 calls of --n keys and nothing else)")
    ap.add_argument("--bulk-copy", type=int, default=None,
                    help="profile mode: staging mode of the merge rounds (0 plain loads, 1 bulk copies, 2 cp.async, "
                         "3 persistent); default: the library's choice")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve mode: arrivals per second (0: all at once)")
    ap.add_argument("--max-size", type=int, default=1 << 26, help="serve mode: largest request (keys)")
    ap.add_argument("--seconds", type=float, default=60.0, help="serve mode: arrival window")
    ap.add_argument("--segments", type=int, default=50000, help="batched mode: number of arrays")
    args = ap.parse_args()
    if args.steps < 1 or args.warmup < 0:
        ap.error("steps >= 1, warmup >= 0")
    if args.impl == "reference":
        return run_reference(args)
    if args.mode != "sort":
        import torch
        from conftest import Oracle, load_gms_module

        gms = load_gms_module()
        gms.build()
        lib = gms.load()
        orc = Oracle()
        if args.mode == "profile":
            return profile_run(lib, orc, args)
        if args.mode == "trace":
            res = host_trace(lib, gms, orc, args.n, args.warmup, args.trace_out)
        elif args.mode == "batched":
            res = batched_bench(lib, orc, total_keys=None, nseg=args.segments)
        else:
            res = serving_bench(lib, orc, seconds=args.seconds, rate=args.rate, hi=args.max_size)
        print(json.dumps({"mode": args.mode, **res}), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
