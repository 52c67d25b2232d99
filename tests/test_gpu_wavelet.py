"""Block-level wavelet transforms on the GPU against the oracle: the
one-level FWT (spaghetti order), the IWT and WC thresholding are
bit-identical; IWT(FWT(u)) reproduces u (the reference's invertibility unit
test, LIB/TESTING/unit_test_waveletDecomposition.f90:47-171, run on the
device)."""
import numpy as np
import pytest

from helpers import random_state, small_cfg, smooth_state
from pyoracle import Oracle, interior
from wabbit_gb300 import config, grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

CASES = [(2, "CDF40"), (2, "CDF44"), (2, "CDF22"), (2, "CDF62"), (3, "CDF40"), (3, "CDF44")]


def _cfg(dim, wavelet):
    g, _ = config.wavelet_ghosts(wavelet)
    Bs = 8 if 2 * g - 1 <= 8 else 12
    return small_cfg(dim, wavelet, Bs=Bs, jmin=1 if dim == 3 else 2, jmax=2 if dim == 3 else 4)


@pytest.mark.parametrize("dim,wavelet", CASES)
def test_decompose_reconstruct_threshold_bitexact(dim, wavelet):
    cfg = _cfg(dim, wavelet)
    # velocity thresholded as a group, pressure on its own (component flag 1
    # is skipped by wc_threshold_tree)
    for c in range(cfg.neq):
        cfg.threshold_state_vector_component[c] = 2 if c < dim else 0
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=13, frac=0.3)
    o = Oracle(cfg)
    o.set_grid(lv, co, smooth_state(cfg, lv, co, 31))
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    synced = o.data()
    wd = o.fwt()
    o.set_data(wd)
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    wd_synced = o.data()
    rec = o.iwt(wd_synced)
    iw = np.abs(interior(cfg, wd))
    th = 0.5 * iw.max(axis=tuple(k for k in range(iw.ndim) if k != 1))
    wdt = o.wc_threshold(wd_synced, th)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(synced)
        _, det0 = f.coarseningIndicator(np.full(cfg.neq, 1.0))
        eps = np.median(det0, axis=0)
        fl_ref, det_ref = f.coarseningIndicator(eps)
        f.wavelet_decompose()
        assert np.array_equal(interior(cfg, f.download()), interior(cfg, wd))
        # the indicator read from the decomposed state gives the same flags
        fl, det = f.coarseningIndicator(eps, input_is_wd=True)
        assert np.array_equal(fl, fl_ref) and np.array_equal(det, det_ref)
        assert (fl == -1).any() and (fl == 0).any()
        f.upload(wd_synced)
        f.wavelet_reconstruct()
        assert np.array_equal(interior(cfg, f.download()), interior(cfg, rec))
        f.upload(wd_synced)
        f.wc_threshold(th)
        got = f.download()
        assert np.array_equal(got, wdt)
        assert (interior(cfg, got) == 0).sum() > (interior(cfg, wd_synced) == 0).sum()


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (2, "CDF44"), (3, "CDF44")])
def test_device_invertibility(dim, wavelet):
    cfg = small_cfg(dim, wavelet, Bs=16, jmin=2 if dim == 2 else 1, jmax=2 if dim == 2 else 1)
    lv, co = grids.equidistant(dim, cfg.Jmin)
    u = random_state(cfg, len(lv), 3)
    with Context(cfg, len(lv) + 2) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(u)
        f.sync_ghosts_tree()
        ref = interior(cfg, f.download())
        f.wavelet_decompose()
        f.sync_ghosts_tree()
        f.wavelet_reconstruct()
        got = interior(cfg, f.download())
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-14
