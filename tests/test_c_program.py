"""A plain C host of the C ABI: tests/c/main_loop.c, compiled by the system C
compiler against include/wabbit_gb300.h alone and linked with the library,
runs the reference's main loop (sync, refine everywhere, RK4 steps, adapt;
LIB/MAIN/main.f90:309-427) and checks every status, the adapted grids and
the state."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "main_loop.c")


def compile_program(tmp_path):
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    from wabbit_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "main_loop")
    # the CUDA runtime the library needs is resolved when the program runs
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lwabbit_gb300", f"-Wl,-rpath,{libdir}", "-Wl,--allow-shlib-undefined", "-lm",
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def cuda_lib_dirs():
    from wabbit_gb300 import build
    root = os.path.dirname(os.path.dirname(os.path.realpath(build.nvcc())))
    out = [os.path.join(root, "lib64"), os.path.join(root, "lib")]
    try:
        import torch
        out.append(os.path.join(os.path.dirname(torch.__file__), "lib"))
    except ImportError:
        pass
    return [d for d in out if os.path.isdir(d)]


def test_c_program_builds(tmp_path):
    assert os.path.exists(compile_program(tmp_path))


@pytest.mark.gpu
def test_c_program_main_loop(tmp_path):
    exe = compile_program(tmp_path)
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = os.pathsep.join(cuda_lib_dirs() + [env.get("LD_LIBRARY_PATH", "")])
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "main loop OK" in r.stdout
    assert r.stdout.count("iteration") == 3
