"""Multi-rank (replica) coordination of bench.py on CPU with gloo, world size 2:
the job time is the maximum over ranks and the job rate counts every rank's
keys; under torchrun the CPU reference arm runs on rank 0 only and prints one
line while the other rank exits 0.  No GPU involved."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = 0.25 * (rank + 1)  # rank 1 is the slow one
        t = bench.max_over_ranks(dist, local, device="cpu")
        rate = bench.job_rate(1 << 20, world, 4, t)
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"t": t, "rate": rate}, f)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    for g in got:
        assert g["t"] == pytest.approx(0.5)
        assert g["rate"] == pytest.approx((1 << 20) * 2 * 4 / 0.5 / 1e9)
    assert bench.max_over_ranks(None, 0.3) == 0.3


def test_reference_arm_under_torchrun(oracle):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--keys", str(1 << 20)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
