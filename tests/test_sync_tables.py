"""Ghost-patch tables (host logic, no GPU): the device sync kernel's
semantics, emulated in numpy over the table, reproduce the oracle's
sequential synchronisation bit for bit, and no patch of a stage reads a
ghost node that the same stage writes (so the stage can run in parallel)."""
import numpy as np
import pytest

import sync_emulator as se
from helpers import random_state, small_cfg
from pyoracle import Oracle
from wabbit_gb300 import build, config, grids


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()


CASES = [("CDF40", 2, 8), ("CDF20", 2, 8), ("CDF60", 2, 16), ("CDF40", 3, 8)]


@pytest.mark.parametrize("wavelet,dim,bs", CASES)
@pytest.mark.parametrize("full", [False, True])
def test_table_emulation_matches_oracle(wavelet, dim, bs, full):
    cfg = small_cfg(dim, wavelet, Bs=bs, jmin=2 if dim == 2 else 1, jmax=4 if dim == 2 else 3)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=4, frac=0.3)
    data = random_state(cfg, len(lv), 1)
    gm = cfg.g if full else cfg.g_rhs
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.sync(gm, gm)
    table = se.host_table(cfg, lv, co, gm, gm)
    got = se.apply(table, data.copy(), int(wavelet[3]))
    assert np.array_equal(got, o.data())


def _written(P):
    w = set()
    for p in P:
        for z in range(p[6], p[9] + 1):
            for y in range(p[5], p[8] + 1):
                for x in range(p[4], p[7] + 1):
                    w.add((p[1], z, y, x))
    return w


@pytest.mark.parametrize("wavelet,dim,bs", CASES + [("CDF44", 2, 12)])
def test_stages_have_no_internal_dependencies(wavelet, dim, bs):
    cfg = small_cfg(dim, wavelet, Bs=bs, jmin=2 if dim == 2 else 1, jmax=5 if dim == 2 else 3)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=9, frac=0.35)
    for gm in (cfg.g_rhs, cfg.g):
        t = se.host_table(cfg, lv, co, gm, gm)
        for st in set(t[:, 3]):
            P = t[t[:, 3] == st]
            w = _written(P)
            assert sum((p[2] - p[2]) for p in P) == 0
            total = sum((p[7] - p[4] + 1) * (p[8] - p[5] + 1) * (p[9] - p[6] + 1) for p in P)
            assert len(w) == total, "two patches of one stage write the same ghost node"
            for p in P:
                if p[2] == 1:
                    for iz in range(p[9] - p[6] + 1):
                        for iy in range(p[8] - p[5] + 1):
                            for ix in range(p[7] - p[4] + 1):
                                k = (p[0], p[12] + 2 * (p[18] + iz), p[11] + 2 * (p[17] + iy), p[10] + 2 * (p[16] + ix))
                                assert k not in w
                elif p[2] == 2:
                    for z in range(p[12], p[15] + 1):
                        for y in range(p[11], p[14] + 1):
                            for x in range(p[10], p[13] + 1):
                                assert (p[0], z, y, x) not in w


def test_invalid_grid_rejected():
    cfg = small_cfg(2, "CDF40", jmin=1, jmax=4)
    lv = np.array([1, 1, 1, 3], np.int32)          # not a complete tree
    co = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [7, 7, 0]], np.int32)
    from wabbit_gb300 import capi
    with pytest.raises(capi.WgError):
        se.host_table(cfg, lv, co, 2, 2)


def test_small_block_with_wide_ghosts_rejected():
    cfg = small_cfg(2, "CDF60", Bs=8, jmin=2, jmax=3)
    lv, co = grids.equidistant(2, 2)
    from wabbit_gb300 import capi
    with pytest.raises(capi.WgError):
        se.host_table(cfg, lv, co, 5, 5)
