"""C-ABI library: builds, loads without a GPU and exports every symbol the
public header declares."""
import ctypes
import os
import re

import pytest

from wabbit_gb300 import build, capi, config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def header_symbols():
    with open(os.path.join(ROOT, "include", "wabbit_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(wg_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(capi.EXPORTS) == syms


def test_config_struct_matches_header(lib):
    c = config.WgConfig()
    assert lib.wg_config_defaults(ctypes.byref(c), 3) == 0
    assert (c.dim, c.neq, c.Bs[2]) == (3, 4, 16)
    assert c.wavelet == b"CDF40"
    # reference default CFL_nu for FD4 in 3-D
    assert abs(c.CFL_nu - 0.95 * 2.79 / (5.333 * 3)) < 1e-15
    assert lib.wg_bytes_per_block(ctypes.byref(c)) > 0


def test_errors_are_returned_not_raised(lib):
    c = config.WgConfig()
    lib.wg_config_defaults(ctypes.byref(c), 2)
    c.neq = 7
    h = ctypes.c_void_p()
    st = lib.wg_ctx_create(ctypes.byref(c), 10, ctypes.byref(h))
    assert st < 0 and not h.value
    assert b"neq" in lib.wg_last_error()
