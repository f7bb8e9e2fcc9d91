"""The testMM-compatible driver (gpu-mms_gb300/testmm): same usage line and
output format as the reference's ./testMM <N> (src/testMM.cu:49-63,192,210-212),
so its sweep scripts run unchanged."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_usage_line(gms):
    r = subprocess.run([gms.CLI], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.strip() == "Usage: ./testMM <N>"


@pytest.mark.parametrize("n", [1, 1000, 1048576 + 9000, 4154368])
def test_output_format_and_sorted(gms, n):
    r = subprocess.run([gms.CLI, str(n)], capture_output=True, text=True, timeout=300)
    lines = r.stdout.strip().splitlines()
    assert re.fullmatch(r"[0-9.]+ [0-9.]+ [0-9.]+", lines[0]), lines
    assert lines[1] == "SORTED!", lines
