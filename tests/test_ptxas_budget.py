"""Register and spill budget of the hot kernels, from ptxas's own report.

The merge kernels are compiled for the CTAs per SM that their shared memory
allows (MergeMinBlocks launch bounds); when the compiler was left to choose,
one source change moved the persistent float32 + int32 merge from 72 to 92
registers (two CTAs per SM instead of three, +16% sort time) and another held
the 32-bit keys-only merge to 40 registers with spills (+21% merge time),
both without any change in results.  This test compiles the translation
units that hold the data-round and base-case kernels (sm_103a, as build()
does) and checks, per instantiation, that nothing spills and that the
registers of the intended CTAs per SM fit the 64K register file.  CPU only:
nvcc cross-compiles here.
"""
import os
import re
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gpu-mms_gb300", "csrc")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
         "-Xcompiler", "-fPIC", "-Xptxas", "-v"]

# kernel name fragment (mangled) -> (threads per CTA, CTAs per SM it must reach)
EXPECT = {
    # 32-bit keys-only data rounds, 288 x 31
    r"merge_tiles_kernelIjNS_5NoValE.*Li288ELi31E": (288, 3),
    # 64-bit keys-only data rounds, 256 x 17
    r"merge_tiles_kernelImNS_5NoValE.*Li256ELi17E": (256, 3),
    # float32 / int32 keys + int32 payload data rounds, 288 x 15
    r"merge_tiles_kernelIjiNS_7KeyLess.*Li288ELi15E": (288, 3),
    # uint64 keys + int32 payload data rounds, 288 x 15 (two by shared memory)
    r"merge_tiles_kernelImiNS_7KeyLess.*Li288ELi15E": (288, 2),
    # warp-shuffle base cases (three 70 KB CTAs per SM)
    r"base_warp_kernelIjNS_7KeyLess": (256, 3),
    r"base_warp_kernelImNS_7KeyLess": (256, 3),
}


def _ptxas_report(unit):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not available")
    out = os.path.join("/tmp", f"ptxas_budget_{os.getpid()}_{unit}.o")
    r = subprocess.run([NVCC] + FLAGS + ["-c", os.path.join(CSRC, unit), "-o", out], capture_output=True, text=True)
    if os.path.exists(out):
        os.unlink(out)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stderr


def _entries(report):
    """(mangled name, registers, spill store bytes, spill load bytes) per kernel."""
    res = []
    name = None
    spill = (0, 0)
    for line in report.splitlines():
        m = re.search(r"Compiling entry function '([^']+)'", line)
        if m:
            name, spill = m.group(1), (0, 0)
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and name:
            spill = (int(m.group(1)), int(m.group(2)))
            continue
        m = re.search(r"Used (\d+) registers", line)
        if m and name:
            res.append((name, int(m.group(1)), spill[0], spill[1]))
            name = None
    return res


@pytest.fixture(scope="module")
def entries():
    units = ["gms_capi_k32.cu", "gms_capi_k64.cu", "gms_capi_kv.cu"]
    with ThreadPoolExecutor(len(units)) as ex:
        reports = list(ex.map(_ptxas_report, units))
    out = []
    for rep in reports:
        out += _entries(rep)
    return out


@pytest.mark.parametrize("pattern", sorted(EXPECT))
def test_hot_kernels_fit_their_residency_without_spills(entries, pattern):
    nt, ctas = EXPECT[pattern]
    hits = [e for e in entries if re.search(pattern, e[0])]
    assert hits, f"no kernel matches {pattern}"
    for name, regs, st, ld in hits:
        assert st == 0 and ld == 0, f"{name}: {st} / {ld} bytes of spill stores / loads"
        assert regs * nt * ctas <= 65536, f"{name}: {regs} registers x {nt} threads x {ctas} CTAs > 64K"
