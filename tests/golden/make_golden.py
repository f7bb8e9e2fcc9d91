"""Regenerates tests/golden/ref_random_list.npz from the reference itself.

Runs oracle/_ref/ref_pin (built by `make -C oracle ref` from the GPU-MMS
sources) which calls the reference's own create_random_list after srand(seed)
(src/buildData.h:54-65, src/testMM.cu:156), its selection_sort<int,host_cmp>
over the whole array (src/testMM.cu:308-320) and the per-tile selection sort
that test_squareSort uses to check the base case (src/testMM.cu:264-269).

The fixture pins the CPU oracle (oracle/oracle.cpp) and is the golden input /
output set for the GPU parity tests.  Usage: python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PIN = os.path.join(ROOT, "oracle", "_ref", "ref_pin")

# (n, seed): seed 0 is the seed testMM uses; sizes straddle the reference's
# M=1024 tile and this library's base tile and bracket its edge cases.
CASES = [(0, 0), (1, 0), (2, 0), (31, 0), (1000, 0), (1023, 0), (1024, 0), (1025, 0),
         (2048, 0), (3000, 1), (4097, 2), (8704, 0), (9000, 3), (12345, 7), (20000, 0)]


def main():
    if not os.path.exists(PIN):
        sys.exit("oracle/_ref/ref_pin missing: run `make -C oracle ref` where the reference is present")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for n, seed in CASES:
            path = os.path.join(td, f"{n}_{seed}.bin")
            subprocess.run([PIN, str(n), str(seed), path], check=True)
            raw = open(path, "rb").read()
            nn = int(np.frombuffer(raw[:8], dtype=np.int64)[0])
            assert nn == n
            arr = np.frombuffer(raw[8:], dtype=np.int32)
            out[f"in_{n}_{seed}"] = arr[:n].copy()
            out[f"sorted_{n}_{seed}"] = arr[n:2 * n].copy()
            out[f"tiles1024_{n}_{seed}"] = arr[2 * n:3 * n].copy()
    out["cases"] = np.array(CASES, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_random_list.npz"), **out)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
