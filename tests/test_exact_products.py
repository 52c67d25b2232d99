"""Integer-pipe tap products (wabbit_gb300/csrc/exact.cuh) against the host's
IEEE multiply: the header compiles for the host, and a C++ program checks
millions of products (random bit patterns, normal ranges, significands with
long runs of low zero or one bits for ties and carries) for bit identity, and
that the fallback flag is raised only at subnormal, special or out-of-range
inputs and results."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "wabbit_gb300", "csrc")


def test_exact_tap_products_match_ieee_multiply(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "exact_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "exact_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe, "1000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = r.stdout.split()
    assert fields[fields.index("failures") + 1] == "0"
    # every CDF4,4 / CDF4,0 tap and the 4th-order interpolation weights take
    # the integer pipe (kinds 1-3); only 0.1 and the 8th-order 245/2048 and
    # 1225/2048 fall back
    k = fields.index("kinds")
    kinds = [int(v) for v in fields[k + 1:k + 5]]
    assert kinds[0] == 6 and sum(kinds) == 44
