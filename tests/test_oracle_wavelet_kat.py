"""Known-answer tests of the oracle's wavelet transforms (no GPU): the
reference's invertibility unit test (LIB/TESTING/unit_test_waveletDecomposition.f90:
47-171: equidistant grid, random data, FWT of every block, ghost sync of the
decomposed data, IWT, relative L2 error of IWT(FWT(u)) - u) and the
semantics of wc_threshold_tree."""
import numpy as np
import pytest

from helpers import random_state, small_cfg
from pyoracle import Oracle, interior
from wabbit_gb300 import config, grids


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF20"), (2, "CDF22"), (2, "CDF40"), (2, "CDF42"), (2, "CDF44"),
                                         (2, "CDF60"), (2, "CDF62"), (3, "CDF40"), (3, "CDF44")])
def test_iwt_of_fwt_is_identity(dim, wavelet):
    g, _ = config.wavelet_ghosts(wavelet)
    Bs = 16 if (dim == 2 or 2 * g - 1 > 8) else 8
    cfg = small_cfg(dim, wavelet, Bs=Bs, jmin=2 if dim == 2 else 1, jmax=2 if dim == 2 else 1)
    lv, co = grids.equidistant(dim, cfg.Jmin)
    o = Oracle(cfg)
    o.set_grid(lv, co, random_state(cfg, len(lv), 5))
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    u = o.data()
    o.set_data(o.fwt())
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    r = o.iwt(o.data())
    err = np.linalg.norm(interior(cfg, r) - interior(cfg, u)) / np.linalg.norm(interior(cfg, u))
    assert err < 1e-14, err


def test_wc_threshold_semantics():
    cfg = small_cfg(2, "CDF44", Bs=16, jmin=2, jmax=2)
    cfg.threshold_state_vector_component[:3] = (2, 2, 0)
    lv, co = grids.equidistant(2, 2)
    o = Oracle(cfg)
    o.set_grid(lv, co, random_state(cfg, len(lv), 9))
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    wd = o.fwt()
    th = np.array([0.3, 0.3, 0.5])
    out = o.wc_threshold(wd, th)
    g = cfg.g
    ii = interior(cfg, wd)
    oo = interior(cfg, out)
    sc = np.zeros(ii.shape[-2:], bool)
    sc[::2, ::2] = True                       # first interior point is an SC
    # SC untouched, ghosts untouched
    assert np.array_equal(ii[..., sc], oo[..., sc])
    mask_g = np.ones(wd.shape, bool)
    mask_g[..., g:-g, g:-g] = False
    assert np.array_equal(wd[mask_g], out[mask_g])
    # component 2 (group 0): zeroed where |WC| < its threshold, kept otherwise
    wc2 = ii[:, 2][:, ~sc]
    assert np.all(oo[:, 2][:, ~sc][np.abs(wc2) < 0.5] == 0.0)
    assert np.array_equal(oo[:, 2][:, ~sc][np.abs(wc2) >= 0.5], wc2[np.abs(wc2) >= 0.5])
    # group 2 (velocity): each component individually, then by the group norm
    u, v = ii[:, 0][:, ~sc], ii[:, 1][:, ~sc]
    keep = (np.sqrt(u * u + v * v) >= 0.3)
    for c, a in ((0, u), (1, v)):
        exp = np.where((np.abs(a) < 0.3) | ~keep, 0.0, a)
        assert np.array_equal(oo[:, c][:, ~sc], exp)
