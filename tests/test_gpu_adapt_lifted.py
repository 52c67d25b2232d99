"""Grid adaptation with lifted wavelets (CDF44: full-tree FWT with coarse
extension, filtered restriction, security zone, reconstruction at the
coarse/fine interfaces; LIB/MESH/adapt_tree.f90:11-255) on the GPU: grid and
state equal the oracle's bit for bit, including the ghost nodes of the final
filtered sync."""
import numpy as np
import pytest

from helpers import small_cfg, smooth_state
from pyoracle import Oracle, interior, pad_blocks
from wabbit_gb300 import config, grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _sorted(lv, co, u):
    order = np.lexsort((co[:, 0], co[:, 1], co[:, 2], lv))
    return lv[order], co[order], u[order]


@pytest.mark.parametrize("w,src", [("CDF44", "CDF40"), ("CDF42", "CDF40"), ("CDF62", "CDF60")])
def test_coarsen_everywhere_cdf44_matches_oracle(golden, w, src):
    """The lifted adaptation everywhere on the file refined with the
    wavelet's predictor: bit for bit the oracle's, and within 4e-15 of
    TESTING/wavelets/adaptive_<w>/vor_00200.h5 (the CE zones of these
    wavelets are wider than the FD stencil, so the widening the device's
    set-up applies changes nothing)."""
    z = golden("wavelet_adaptive.npz")
    cfg = config.defaults(2)
    cfg.Bs[0] = cfg.Bs[1] = 32
    cfg.domain[0] = cfg.domain[1] = 6.283185307179586
    cfg.wavelet = w.encode()
    cfg.g, cfg.g_rhs = config.wavelet_ghosts(w)[0], 2
    cfg.Jmin, cfg.Jmax = 1, 7
    key = "refined" if src == "CDF40" else f"refined_{src}"
    u1 = z[f"{key}_u"]
    u3 = np.concatenate([u1, 0.5 * u1 ** 2, -u1], axis=1)
    data = pad_blocks(cfg, u3)
    o = Oracle(cfg)
    o.set_grid(z[f"{key}_level"], z[f"{key}_coords"], data)
    o.sync(cfg.g, cfg.g, ignore_filter=False)
    assert o.adapt(everywhere=True) == 112
    with Context(cfg, 2 * len(u1)) as ctx:
        f = ctx.forest()
        f.set_grid(z[f"{key}_level"], z[f"{key}_coords"])
        f.upload(data)
        assert f.adapt(everywhere=True) == 112
        b = _sorted(*f.grid(), f.download())
    a = _sorted(*o.grid(), o.data())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2])
    assert np.array_equal(a[0], z[f"coarsened_{w}_level"])
    assert np.abs(interior(cfg, b[2])[:, :1] - z[f"coarsened_{w}_u"]).max() <= 4e-15


@pytest.mark.parametrize("dim,Bs,jmin,jmax,quantile", [(2, 32, 1, 4, 0.6), (2, 16, 2, 5, 0.5), (3, 16, 1, 3, 0.8),
                                                      (2, 16, 2, 7, 0.5), (3, 16, 1, 4, 0.7)])
def test_threshold_adapt_cdf44_matches_oracle(dim, Bs, jmin, jmax, quantile):
    """Bs=32 takes the leaf-first decomposition and the leaf-only
    reconstruction; Bs=16 (below 3 x the HD half-width and below Ndep2r)
    the level-wise decomposition and reconstruction. The Jmax=7 grid (2,218
    leaves, ~2,900 full-tree blocks) is planned on the host thread pool, and
    its copy/restriction stages are waves made of per-chunk lists; on it and
    on the four-level 3-D grid the level-wise reconstruction reads blocks
    reconstructed at the level below from hvy_tmp."""
    cfg = small_cfg(dim, "CDF44", Bs=Bs, jmin=jmin, jmax=jmax)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=33, frac=0.45)
    data = smooth_state(cfg, lv, co, 9)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    _, det = o.flags(np.full(cfg.neq, 1.0))
    eps = np.quantile(det, quantile, axis=0)
    with Context(cfg, 2 * len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        for rnd in range(2):
            o.sync(cfg.g, cfg.g, ignore_filter=False)
            n_ref = o.adapt(eps)
            n = f.adapt(eps)
            assert n == n_ref
            a = _sorted(*o.grid(), o.data())
            b = _sorted(*f.grid(), f.download())
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            assert np.array_equal(a[2], b[2])
            eps = eps * 4.0
        assert n < len(lv)
