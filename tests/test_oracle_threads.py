"""The oracle gives the same bits with one thread and with many: ghost syncs
(unfiltered and, for lifted wavelets, filtered), the RHS, RK4 steps with a
sparse mask, and the interior upload, on graded grids with level jumps in 2-D
and 3-D. The multi-threaded oracle is what the CPU baseline times."""
import numpy as np
import pytest

from helpers import small_cfg, smooth_state, sphere_mask
from pyoracle import Oracle, interior
from wabbit_gb300 import grids


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (2, "CDF44"), (3, "CDF40"), (3, "CDF44")])
def test_threads_bit_identical(dim, wavelet):
    cfg = small_cfg(dim, wavelet, Bs=8, penal=1, jmin=1, jmax=3 if dim == 3 else 4)
    cfg.C_eta = 1e-2
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=11, frac=0.4)
    data = smooth_state(cfg, lv, co, 7)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.3) if dim == 3 else None
    out = []
    for threads in (1, 8):
        o = Oracle(cfg, threads=threads)
        o.set_grid(lv, co, data)
        if mask is not None:
            ids = np.nonzero(mask[:, 0].reshape(len(lv), -1).max(axis=1) > 0)[0]
            o.set_mask_sparse(ids, mask[ids])
        res = []
        o.sync(cfg.g_rhs, cfg.g_rhs)
        res.append(o.data())
        if wavelet == "CDF44":
            o.sync(cfg.g, cfg.g, ignore_filter=False)
            res.append(o.data())
        o.set_data(data)
        t = 0.0
        for _ in range(2):
            t, dt = o.step(t)
        res.append(o.data())
        res.append(np.array([t, dt]))
        o.set_interior(interior(cfg, data))
        res.append(o.data())
        out.append(res)
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_sparse_mask_equals_dense():
    """A sparse mask (listed blocks, zeros elsewhere) steps like the dense
    mask array with zeros on the other blocks."""
    cfg = small_cfg(3, "CDF40", Bs=8, penal=1, jmin=1, jmax=3)
    cfg.C_eta = 1e-2
    lv, co = grids.random_graded(3, 1, 3, seed=4, frac=0.4)
    data = smooth_state(cfg, lv, co, 3)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.3)
    ids = np.nonzero(mask[:, 0].reshape(len(lv), -1).max(axis=1) > 0)[0]
    assert 0 < len(ids) < len(lv)
    res = []
    for sparse in (False, True):
        o = Oracle(cfg, threads=4)
        o.set_grid(lv, co, data)
        if sparse:
            o.set_mask_sparse(ids, mask[ids])
        else:
            o.set_mask(mask)
        o.step(0.0)
        res.append((o.data(), o.mask()))
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
