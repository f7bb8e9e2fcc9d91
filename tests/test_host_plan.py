"""Host plans of the host-to-host sorts (gms_host_plan.h), compiled with g++
and checked on the CPU: the input chunk boundaries (every interior boundary
on a unit of k^q base tiles, so q merge rounds run chunk by chunk; a small
first and last chunk) and the parts of the last merge round."""
import os
import random
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gpu-mms_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include "gms_host_plan.h"
int main() {
  char op;
  long long a, b, c;
  while (scanf(" %c %lld %lld %lld", &op, &a, &b, &c) == 4) {
    int64_t out[gms::kMaxParts + gms::kHostChunks + 1];
    int n = op == 'C' ? gms::host_chunk_plan(a, (int)b, (int)c, out) : gms::host_split_ends(a, (int)b, c != 0, out);
    printf("%d", n);
    for (int i = 0; i < (op == 'C' ? n + 1 : n); ++i) printf(" %lld", (long long)out[i]);
    printf("\n");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def plan_exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("host_plan")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def run(exe, queries):
    text = "\n".join(" ".join(str(x) for x in q) for q in queries) + "\n"
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split("\n")
    res = []
    for line in out[: len(queries)]:
        v = [int(x) for x in line.split()]
        res.append(v[1:])
    return res


def unit_of(tiles, k, passes):
    unit, q = 1, 0
    while q < passes - 1 and unit * k * 8 <= tiles:
        unit *= k
        q += 1
    return unit


def test_chunk_plan_int32_2p28(plan_exe):
    # 2^28 keys: 32768 base tiles of 8192, k = 32, three merge rounds
    (start,) = run(plan_exe, [("C", 32768, 32, 3)])
    sizes = [b - a for a, b in zip(start, start[1:])]
    assert [s // 1024 for s in sizes] == [1, 1, 2, 3, 4, 4, 4, 4, 3, 3, 2, 1]


def test_chunk_plan_invariants(plan_exe):
    rng = random.Random(3)
    queries = []
    for _ in range(4000):
        k = rng.choice([2, 3, 8, 16, 32])
        tiles = rng.choice([rng.randint(1, 64), rng.randint(1, 5000), rng.randint(1, 1 << 22)])
        passes = rng.randint(0, 6)
        queries.append(("C", tiles, k, passes))
    queries += [("C", 1, 32, 0), ("C", 2, 32, 1), ("C", 8192, 32, 3), ("C", 16384, 32, 3), ("C", 1 << 18, 32, 4)]
    for (_, tiles, k, passes), start in zip(queries, run(plan_exe, queries)):
        n = len(start) - 1
        assert 1 <= n <= 16
        assert start[0] == 0 and start[-1] == tiles
        assert all(a < b for a, b in zip(start, start[1:]))
        unit = unit_of(tiles, k, passes)
        assert all(s % unit == 0 for s in start[1:-1]), (tiles, k, passes, start)
        sizes = [-(-(b - a) // unit) for a, b in zip(start, start[1:])]
        if n > 1:
            assert sizes[0] == 1
        # rising, then falling (a plateau allowed; the last chunk may be short)
        peak = sizes.index(max(sizes[:-1] or sizes))
        assert all(a <= b for a, b in zip(sizes[:peak], sizes[1:peak + 1])), sizes
        units = -(-tiles // unit)
        if units >= 16:
            assert sizes[-1] == 1 and max(sizes) >= 2
            assert all(a >= b for a, b in zip(sizes[peak:-1], sizes[peak + 1:])), sizes


def test_split_ends(plan_exe):
    rng = random.Random(4)
    queries = [("S", rng.randint(1, 1 << 20), rng.randint(1, 70), rng.randint(0, 1)) for _ in range(3000)]
    queries += [("S", 36864, 8, 1), ("S", 63, 8, 1), ("S", 64, 8, 1), ("S", 5, 8, 0), ("S", 1, 1, 1)]
    for (_, tiles, parts, ramp), ends in zip(queries, run(plan_exe, queries)):
        assert 1 <= len(ends) <= min(max(parts, 1), 64)
        assert ends[-1] == tiles
        assert all(0 < e <= tiles for e in ends)
        assert all(a <= b for a, b in zip(ends, ends[1:]))
        if ramp and min(parts, 64) >= 3 and tiles >= 64:
            assert ends[0] == -(-tiles // 32)
            assert ends[1] == ends[0] + -(-tiles // 16)
    (ends,) = run(plan_exe, [("S", 36864, 8, 1)])
    assert ends[:2] == [1152, 3456] and ends[-1] == 36864 and len(ends) == 8
