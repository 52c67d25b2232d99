"""The host thread pool of the planning code (wabbit_gb300/csrc/par.hpp):
a C++ program checks that every index of thousands of jobs runs exactly once,
that nested calls run inline, that callers on several threads take turns and
that a forked child gets a working pool."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "wabbit_gb300", "csrc")


def test_host_pool(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "par_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "par_check.cpp"), "-o", exe, "-pthread"],
                   check=True, capture_output=True, text=True)
    for _ in range(3):
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0 and "pool failures 0" in r.stdout, r.stdout + r.stderr
