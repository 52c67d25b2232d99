"""Build the CUDA library libwabbit_gb300.so in-tree (wabbit_gb300/_lib/).

Every translation unit is compiled for sm_103a only, in parallel, and linked
with nvcc; no CMake, no torch extension machinery. The strict ACM variant is
compiled with -fmad=false (reference arithmetic, bit-identical results), the
others with FMA contraction. The FMA-throughput probe the benchmark uses as
its ALU denominator is a separate library, libwg_probe.so, so that the
product library holds only the hot path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libwabbit_gb300.so")
PROBE_LIB = os.path.join(OUT_DIR, "libwg_probe.so")
PROBE_SRC = "k_probe.cu"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "forest.cpp": [],
    "geometry.cpp": ["-Xcompiler", "-ffp-contract=off"],
    "adapt.cpp": [],
    "lifted.cpp": [],
    "k_lifted.cu": ["-fmad=false"],
    "capi.cu": [],
    "k_sync.cu": ["-fmad=false"],
    "k_misc.cu": [],
    "k_wavelet.cu": [],
    "k_acm_strict.cu": ["-fmad=false"],
    "k_acm_fast.cu": [],
    "k_acm_df.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC) if f != PROBE_SRC]
    deps.append(os.path.join(HERE, "..", "include", "wabbit_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", SRC] + ARCH


def build_probe(force: bool = False) -> str:
    """The FMA-throughput probe library (measurement only)."""
    src = os.path.join(SRC, PROBE_SRC)
    if not force and os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= os.path.getmtime(src):
        return PROBE_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = PROBE_LIB + ".tmp"
    r = subprocess.run([nvcc()] + COMMON + ["-shared", src, "-o", tmp, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {PROBE_SRC}:\n{r.stderr}")
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    common = COMMON

    def compile_one(item):
        src, extra = item
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [cc] + common + extra + ["-c", os.path.join(SRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_probe(force=True))
