"""The plan of a batched (segmented) sort (gpu-mms_gb300/csrc/gms_seg_plan.h),
compiled with g++ and checked on the CPU:

  * base-case tiles cover every array exactly, none crosses an array's end;
  * round p holds exactly the arrays that need p or more rounds; its groups
    cover each such array with k runs of base * k^(p-1) keys, and a group's
    input runs are the array's units of the level below (tiles or groups),
    numbered consecutively;
  * the buffer flags make every array's writes alternate so that its last
    step (base case or last round) writes the output, and every round reads
    the buffer its array's previous step wrote; exactly the last step decodes;
  * tile and row maps agree with each group's first tile and row, and sample
    levels list each group's block sample where the producers write it.
"""
import os
import random
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gpu-mms_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "gms_seg_plan.h"
int main() {
  long long base, capd, capwd, capi, capwi; int k, b, nseg;
  while (scanf("%lld %lld %lld %lld %lld %d %d %d", &base, &capd, &capwd, &capi, &capwi, &k, &b, &nseg) == 8) {
    std::vector<int64_t> off(nseg + 1);
    for (int i = 0; i <= nseg; ++i) { long long x; scanf("%lld", &x); off[i] = x; }
    gms::SegGeom g{base, capd, capwd, capi, capwi, k, b, 8};
    gms::SegPlanH P = gms::seg_plan(off.data(), nseg, g);
    printf("plan %d %d %zu %zu\n", P.ok ? 1 : 0, P.rounds_max, P.base.size(), P.levels.size());
    for (auto& t : P.base) printf("b %lld %lld %lld %lld\n", (long long)t.start, (long long)t.len, (long long)t.run0, (long long)t.flags);
    for (int r : P.rounds) printf("r %d\n", r);
    for (auto& l : P.levels) {
      printf("l %d %lld %lld %lld %d %d %zu %zu %zu\n", l.depth, (long long)l.n, (long long)l.L, (long long)l.runs,
             l.whole ? 1 : 0, l.sample, l.grp.size(), l.tile_grp.size(), l.row_grp.size());
      for (auto& x : l.grp) printf("g %lld %lld %lld %lld %lld %lld\n", (long long)x.start, (long long)x.len,
                                   (long long)x.run0, (long long)x.tile0, (long long)x.row0, (long long)x.flags);
      printf("t"); for (int v : l.tile_grp) printf(" %d", v); printf("\n");
      printf("w"); for (int v : l.row_grp) printf(" %d", v); printf("\n");
      printf("u"); for (int v : l.run_len) printf(" %d", v); printf("\n");
    }
    printf("end\n");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def plan_exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("seg_plan")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def ceil(a, b):
    return (a + b - 1) // b


def run_plan(exe, geom, off):
    base, capd, capwd, capi, capwi, k, b = geom
    inp = f"{base} {capd} {capwd} {capi} {capwi} {k} {b} {len(off) - 1}\n" + " ".join(map(str, off)) + "\n"
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    it = iter(out)
    head = next(it).split()
    plan = {"ok": head[1] == "1", "R": int(head[2]), "base": [], "rounds": [], "levels": []}
    for _ in range(int(head[3])):
        plan["base"].append(tuple(map(int, next(it).split()[1:])))
    for _ in range(plan["R"]):
        plan["rounds"].append(int(next(it).split()[1]))
    for _ in range(int(head[4])):
        f = next(it).split()
        lv = {"depth": int(f[1]), "n": int(f[2]), "L": int(f[3]), "runs": int(f[4]), "whole": f[5] == "1",
              "sample": int(f[6]), "grp": []}
        for _ in range(int(f[7])):
            lv["grp"].append(tuple(map(int, next(it).split()[1:])))
        lv["tile_grp"] = list(map(int, next(it).split()[1:]))
        lv["row_grp"] = list(map(int, next(it).split()[1:]))
        lv["run_len"] = list(map(int, next(it).split()[1:]))
        plan["levels"].append(lv)
    assert next(it) == "end"
    return plan


def check_levels(plan, lv_i, geom, run_starts=None):
    """Tile/row maps of one level and, recursively, its sample levels."""
    base, capd, capwd, capi, capwi, k, b = geom
    lv = plan["levels"][lv_i]
    grp = lv["grp"][:-1]
    tot = lv["grp"][-1]
    idx = lv["depth"] > 0
    cap, capw = (capi, capwi) if idx else (capd, capwd)
    assert lv["whole"] == (k * lv["L"] <= cap)
    if lv["whole"]:
        assert lv["sample"] == -1 and lv["tile_grp"] == [] and lv["row_grp"] == []
        return
    Ls = ceil(lv["L"], b)
    Gt = capw // b - k
    tile = row = 0
    for g, (start, ln, run0, tile0, row0, fl) in enumerate(grp):
        kg = ceil(ln, lv["L"])
        last = ln - (kg - 1) * lv["L"]
        assert lv["run_len"][run0:run0 + kg] == [lv["L"]] * (kg - 1) + [last]
        ns = (kg - 1) * Ls + ceil(last, b)
        tiles = ceil(ns, Gt)
        assert (tile0, row0) == (tile, row)
        assert lv["tile_grp"][tile:tile + tiles] == [g] * tiles
        assert lv["row_grp"][row:row + tiles + 1] == [g] * (tiles + 1)
        tile += tiles
        row += tiles + 1
    assert tot[3:5] == (tile, row) and len(lv["tile_grp"]) == tile and len(lv["row_grp"]) == row
    # the sample level: group g's block sample, Ls per run, from run0 * Ls
    sl = plan["levels"][lv["sample"]]
    assert sl["depth"] == lv["depth"] + 1 and sl["L"] == Ls and sl["runs"] == lv["runs"]
    assert sl["n"] == lv["runs"] * Ls
    for (start, ln, run0, *_), (s_start, s_len, s_run0, *_) in zip(grp, sl["grp"][:-1]):
        kg = ceil(ln, lv["L"])
        last = ln - (kg - 1) * lv["L"]
        assert (s_start, s_len, s_run0) == (run0 * Ls, (kg - 1) * Ls + ceil(last, b), run0)
    check_levels(plan, lv["sample"], geom)


def check_plan(plan, off, geom):
    base, capd, capwd, capi, capwi, k, b = geom
    assert plan["ok"]
    nseg = len(off) - 1
    lens = [off[s + 1] - off[s] for s in range(nseg)]
    R = []
    for ln in lens:
        p, L = 0, base
        while L < ln:
            L *= k
            p += 1
        R.append(p)
    assert plan["R"] == max(R + [0])
    # base tiles
    units = {}  # segment -> list of (start, len) of its units at the current level, in index order
    tiles = plan["base"]
    i = 0
    last_buf = {}
    for s in range(nseg):
        u = []
        for t in range(ceil(lens[s], base)):
            start, ln, run0, fl = tiles[i]
            assert run0 == i and start == off[s] + t * base and ln == min(base, lens[s] - t * base)
            buf = "out" if fl & 1 else "tmp"
            assert buf == ("out" if R[s] % 2 == 0 else "tmp")
            assert bool(fl & 2) == (R[s] == 0)
            last_buf[s] = buf
            u.append((i, start, ln))
            i += 1
        units[s] = u
    assert i == len(tiles)
    prev_total = len(tiles)
    for p in range(1, plan["R"] + 1):
        L = base * k ** (p - 1)
        lv = plan["levels"][plan["rounds"][p - 1]]
        assert lv["depth"] == 0 and lv["L"] == L and lv["runs"] == prev_total
        grp = lv["grp"][:-1]
        gi = 0
        new_units = {}
        for s in range(nseg):
            if R[s] < p:
                continue
            u = units[s]
            nu = []
            for q in range(ceil(len(u), k)):
                start, ln, run0, tile0, row0, fl = grp[gi]
                chunk = u[q * k:(q + 1) * k]
                assert run0 == chunk[0][0] and [c[0] for c in chunk] == list(range(run0, run0 + len(chunk)))
                assert start == chunk[0][1] == off[s] + q * L * k
                assert ln == sum(c[2] for c in chunk) == min(L * k, lens[s] - q * L * k)
                reads = "out" if fl & 1 else "tmp"
                writes = "tmp" if fl & 1 else "out"
                assert reads == last_buf[s], f"segment {s} round {p} reads the wrong buffer"
                assert bool(fl & 2) == (p == R[s])
                nu.append((gi, start, ln))
                gi += 1
            new_units[s] = nu
            last_buf[s] = writes
        assert gi == len(grp)
        units.update(new_units)
        prev_total = len(grp)
        check_levels(plan, plan["rounds"][p - 1], geom)
    for s in range(nseg):
        if lens[s]:
            assert last_buf[s] == "out", f"segment {s} does not end in the output"


GEOMS = [
    (8192, 8928, 8432, 8704, 8432, 32, 32),   # 32-bit keys only
    (4096, 4352, 4080, 4352, 4080, 32, 32),   # 64-bit keys only
    (4352, 4352, 4080, 4352, 4080, 32, 32),   # key/value
    (64, 96, 80, 96, 80, 4, 8),               # tiny geometry: deep recursion, many rounds
]


@pytest.mark.parametrize("geom", GEOMS)
def test_plans_of_random_batches(plan_exe, geom):
    rng = random.Random(geom[0] * 7 + geom[5])
    base, k = geom[0], geom[5]
    for trial in range(12):
        nseg = rng.randint(1, 40)
        top = base * k ** rng.randint(0, 3)
        lens = []
        for _ in range(nseg):
            r = rng.random()
            lens.append(0 if r < 0.15 else rng.randint(1, base) if r < 0.4 else rng.randint(1, top + 7))
        off = [0]
        for ln in lens:
            off.append(off[-1] + ln)
        if off[-1] == 0:
            continue
        check_plan(run_plan(plan_exe, geom, off), off, geom)


def test_plan_edge_batches(plan_exe):
    geom = GEOMS[3]
    base, k = geom[0], geom[5]
    for lens in ([1], [base], [base + 1], [base * k], [base * k + 1], [0, 0, 5, 0], [base * k ** 3 + 3, 1, 0, 2],
                 [base * k * k] * 3):
        off = [0]
        for ln in lens:
            off.append(off[-1] + ln)
        check_plan(run_plan(plan_exe, geom, off), off, geom)


def test_plan_refuses_an_array_past_int32(plan_exe):
    """Run lengths are 32-bit in the plan's device arrays: an array of 2^31
    keys gets no plan (the C ABI reports GMS_ERR_TOO_LARGE), one of 2^31 - 1
    keys in a batch is planned."""
    geom = (8192, 8928, 8432, 8704, 8432, 32, 32)
    base, capd, capwd, capi, capwi, k, b = geom
    inp = f"{base} {capd} {capwd} {capi} {capwi} {k} {b} 2\n0 5 {5 + (1 << 31)}\n"
    out = subprocess.run([plan_exe], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    assert out[0].split()[:3] == ["plan", "0", "0"]
