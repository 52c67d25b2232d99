"""Ghost-sync patch tables (make_sync_table: per-relation templates, built
on the host thread pool) against a sequential construction from make_patch
(sender order, relation order, boxes shifted to the buffer's ghost width,
stage grouping, largest box and prediction shared-memory need), for CDF4,0,
CDF4,4 and CDF2,2, three ghost widths and two buffer widths, on random graded
2-D and 3-D grids."""
import os
import shutil
import subprocess

import pytest

from wabbit_gb300 import grids

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "wabbit_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("stc") / "sync_table_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "sync_table_check.cpp"),
                    os.path.join(CSRC, "forest.cpp"), "-o", exe, "-pthread"], check=True, capture_output=True,
                   text=True)
    return exe


@pytest.mark.parametrize("dim,jmin,jmax,seed", [(2, 2, 5, 3), (2, 2, 7, 5), (3, 1, 3, 7), (3, 2, 5, 8)])
def test_sync_table_build(checker, tmp_path, dim, jmin, jmax, seed):
    lv, co = grids.random_graded(dim, jmin, jmax, seed=seed, frac=0.45)
    path = tmp_path / "grid.txt"
    with open(path, "w") as f:
        f.write(f"{dim} {len(lv)}\n")
        for l, c in zip(lv, co):
            f.write(f"{l} {c[0]} {c[1]} {c[2] if len(c) > 2 else 0}\n")
    r = subprocess.run([checker, str(path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "differing 0" in r.stdout, r.stdout + r.stderr
