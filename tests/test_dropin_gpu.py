"""The header-only drop-in (include/multimergesort.hxx) compiled into a caller
written for GPU-MMS's multimergesort<T,cmp>: default, descending, absolute
value, packed key/value records (including the CASTTYPE-cast testType shape),
fraction and low-32-bit comparators on 64-bit words, 4- and 5-argument forms,
int / unsigned / long long under the default cmp<T> (the keys-only fast
path), up to 2^24 keys, and three host threads calling at once, checked
against std::stable_sort on the host (tests/dropin/dropin_main.cu)."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_dropin_template_program(gms):
    exe = os.path.join(ROOT, "gpu-mms_gb300", "_build", "dropin_test")
    src = os.path.join(ROOT, "tests", "dropin", "dropin_main.cu")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    deps = [src] + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))] + \
        [os.path.join(ROOT, "gpu-mms_gb300", "csrc", f) for f in os.listdir(os.path.join(ROOT, "gpu-mms_gb300", "csrc"))]
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
        cmd = [gms._nvcc(), "-std=c++17", "--expt-relaxed-constexpr", "-O2", "-gencode",
               "arch=compute_103a,code=sm_103a", "-Xcompiler", "-pthread", "-I", os.path.join(ROOT, "include"),
               src, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "DROPIN OK" in r.stdout, r.stdout[-4000:] + r.stderr[-2000:]
