"""Grid adaptation (adapt_tree, unlifted wavelets) on the GPU: the new grid
and the new state must equal the oracle's bit for bit, and the reference's
coarsen-everywhere regression file (TESTING/wavelets/adaptive_CDF40) is
reproduced."""
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


@pytest.mark.parametrize("w", ["CDF40", "CDF20", "CDF60"])
def test_coarsen_everywhere_golden_cdf40(golden, w):
    """The unlifted adaptation on the file refined with the wavelet's own
    predictor against TESTING/wavelets/adaptive_<w>/vor_00200.h5, bit for
    bit."""
    z = golden("wavelet_adaptive.npz")
    cfg = config.defaults(2)
    cfg.Bs[0] = cfg.Bs[1] = 32
    cfg.domain[0] = cfg.domain[1] = 6.283185307179586
    cfg.wavelet = w.encode()
    cfg.g, cfg.g_rhs = max(3, config.wavelet_ghosts(w)[0]), 2
    cfg.Jmin, cfg.Jmax = 1, 7
    key = "refined" if w == "CDF40" else f"refined_{w}"
    u1 = z[f"{key}_u"]                           # one component; the ACM state carries three copies
    u3 = np.repeat(u1, 3, axis=1)
    with Context(cfg, 2 * len(u1)) as ctx:
        f = ctx.forest()
        f.set_grid(z[f"{key}_level"], z[f"{key}_coords"])
        f.upload(pad_blocks(cfg, u3))
        n = f.adapt(everywhere=True)
        assert n == 112
        lv, co = f.grid()
        lv, co, u = _sorted(lv, co, interior(cfg, f.download()))
    assert np.array_equal(lv, z[f"coarsened_{w}_level"])
    assert np.array_equal(co, z[f"coarsened_{w}_coords"])
    for c in range(3):
        assert np.array_equal(u[:, c:c + 1], z[f"coarsened_{w}_u"])


@pytest.mark.parametrize("dim,wavelet,quantile,jmax", [(2, "CDF40", 0.5, 5), (2, "CDF20", 0.7, 5), (2, "CDF60", 0.4, 5),
                                                       (3, "CDF40", 0.95, 3), (2, "CDF40", 0.5, 7),
                                                       (3, "CDF40", 0.8, 4)])
def test_threshold_adapt_matches_oracle(dim, wavelet, quantile, jmax):
    """Jmax=7 (2-D, six levels, ~2,200 leaves) and Jmax=4 (3-D, four levels)
    take the host thread pool and full trees with long level chains."""
    g, _ = config.wavelet_ghosts(wavelet)
    Bs = 16 if dim == 2 else 8
    cfg = small_cfg(dim, wavelet, Bs=Bs, jmin=2 if dim == 2 else 1, jmax=jmax)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=21, frac=0.45)
    data = smooth_state(cfg, lv, co, 7)
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
            n_ref = o.adapt(eps)
            n = f.adapt(eps)
            assert n == n_ref
            a = _sorted(*o.grid(), o.data())
            b = _sorted(*f.grid(), f.download())
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            assert np.array_equal(a[2], b[2])
            eps = eps * 4.0
        assert n < len(lv)


def test_refine_step_adapt_loop_matches_oracle():
    """Three cycles of the reference's main loop with adaptation (refine
    everywhere, RK4 step, adapt; LIB/MAIN/main.f90:314-400) with the
    bit-exact stencil variant."""
    cfg = small_cfg(2, "CDF40", Bs=16, jmin=2, jmax=5)   # blocks reaching Jmax stay when refining
    cfg.eps, cfg.eps_normalized = 1e-6, 0
    lv, co = grids.random_graded(2, 2, 4, seed=3, frac=0.4)
    data = smooth_state(cfg, lv, co, 9)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    eps = np.full(cfg.neq, cfg.eps)
    with Context(cfg, 16 * len(lv)) as ctx:
        ctx.set_variant(False)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_time(0.0)
        t = 0.0
        top = 0
        for cycle in range(3):
            o.sync(cfg.g, cfg.g, ignore_filter=True)
            o.refine_everywhere()
            t, _ = o.step(t)
            n_ref = o.adapt(eps)
            f.sync_ghosts_tree()
            f.refine_everywhere()
            top = max(top, int(f.grid()[0].max()))
            f.timeStep_tree()
            n = f.adapt(eps)
            assert n == n_ref, cycle
            a = _sorted(*o.grid(), o.data())
            b = _sorted(*f.grid(), f.download())
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            assert np.array_equal(interior(cfg, a[2]), interior(cfg, b[2])), cycle
        assert top == cfg.Jmax   # refinement reached Jmax and stayed there


@pytest.mark.gpu
@pytest.mark.parametrize("dim,wavelet,Bs", [(2, "CDF40", 16), (2, "CDF44", 16), (3, "CDF40", 8), (3, "CDF44", 16),
                                            (3, "CDF40", 16)])
def test_refine_everywhere_full_blocks_match_oracle(dim, wavelet, Bs):
    """refine_everywhere (refinementExecute.f90:4-116) on every point of the
    daughters, ghosts included, against the oracle: the separable prediction
    per daughter slab reproduces the parent's full-block prediction. Tiny
    (subnormal) and zero values in one component take the FP64 fallback of
    the integer-pipe products."""
    cfg = small_cfg(dim, wavelet, Bs=Bs, jmin=1 if dim == 3 else 2, jmax=4 if dim == 3 else 6)
    lv, co = grids.random_graded(dim, cfg.Jmin + 1, cfg.Jmax - 1, seed=11, frac=0.4)
    data = smooth_state(cfg, lv, co, 5)
    data[: len(lv) // 3, 0] *= 1e-310          # subnormal products
    data[len(lv) // 3: len(lv) // 2, 1] = 0.0   # signed zeros
    data[len(lv) // 2: 2 * len(lv) // 3, 1] *= -1e300
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.refine_everywhere()
    with Context(cfg, 10 * len(lv)) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.refine_everywhere()
        a = _sorted(*o.grid(), o.data())
        b = _sorted(*f.grid(), f.download())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2].view(np.int64), b[2].view(np.int64))
