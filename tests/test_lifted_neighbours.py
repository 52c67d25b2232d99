"""Neighbour lists of the lifted adaptation's full tree (one all-alive search
filtered per alive set, wabbit_gb300/csrc/lifted.cpp) against a direct
restatement of find_neighbor with search_overlapping, on random graded 2-D
and 3-D trees (small and above the host pool's parallel threshold) and six
alive sets each."""
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
    exe = str(tmp_path_factory.mktemp("lnc") / "lifted_nbr_check")
    srcs = [os.path.join(HERE, "lifted_nbr_check.cpp")] + [os.path.join(CSRC, f) for f in
                                                          ("lifted.cpp", "forest.cpp", "adapt.cpp")]
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC] + srcs + ["-o", exe, "-pthread"], check=True,
                   capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("dim,jmin,jmax,seed", [(2, 2, 5, 1), (2, 2, 7, 33), (3, 1, 3, 2), (3, 2, 5, 4)])
def test_lifted_neighbour_lists(checker, tmp_path, dim, jmin, jmax, seed):
    lv, co = grids.random_graded(dim, jmin, jmax, seed=seed, frac=0.45)
    path = tmp_path / "grid.txt"
    with open(path, "w") as f:
        f.write(f"{dim} {len(lv)}\n")
        for l, c in zip(lv, co):
            f.write(f"{l} {c[0]} {c[1]} {c[2] if len(c) > 2 else 0}\n")
    r = subprocess.run([checker, str(path), str(jmin), str(jmax)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "neighbour mismatches 0" in r.stdout, r.stdout + r.stderr
