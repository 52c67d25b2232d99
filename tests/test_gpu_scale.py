"""Parity at the benchmark configurations' scale (slow GPU tests).

* The adapt path (the 3-D CDF4,4 adapt workload, 16^3 blocks, g = 6,
  eps = 1e-4 x the Linfty norm per component) at Jmax = 5, 9,584 blocks on
  levels 3-5: the coarsening indicator of every leaf, and the adapted tree
  and state (adapt_tree, LIB/MESH/adapt_tree.f90:11-255) with that eps and
  with one that removes about half of the leaves, equal the oracle's bit for
  bit.
* The batched mixed-precision stepper (the penalised-sphere ACM channel,
  CDF4,4, 16^3 blocks) on its Jmax = 5 grid, 3,144 blocks: three RK4 steps
  of the FP32-pipe path through wg_run stay within 1e-10 (relative L2) of
  the FP64 oracle, with the same time.
"""
import numpy as np
import pytest

from pyoracle import Oracle
from wabbit_gb300 import workloads
from wabbit_gb300.solver import Context

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _sorted(lv, co, u):
    order = np.lexsort((co[:, 0], co[:, 1], co[:, 2], lv))
    return lv[order], co[order], u[order]


def test_adapt_workload_jmax5_matches_oracle():
    cfg = workloads.make_config("adapt3d_cdf44")
    cfg.Jmax = 5
    lv, co = workloads.make_grid("adapt3d_cdf44", cfg)
    assert len(lv) == 9584 and list(np.unique(lv)) == [3, 4, 5]
    u = workloads.adapt_field_device(cfg, lv, co)
    un = u.cpu().numpy()
    eps = cfg.eps * np.abs(un).max(axis=(0, 2, 3, 4))
    o = Oracle(cfg, threads=16)
    o.set_grid(lv, co, None)
    o.set_interior(un)
    with Context(cfg, int(len(lv) * 1.2) + 64) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload_interior(u)
        del u
        # the indicator of every leaf (one-level FWT, threshold-state-vector)
        f.sync_ghosts_tree()
        o.sync(cfg.g, cfg.g, ignore_filter=True)
        flags, det = f.coarseningIndicator(eps)
        flags_ref, det_ref = o.flags(eps)
        assert np.array_equal(flags, flags_ref)
        assert np.array_equal(det, det_ref)
        # adapt_tree on the whole tree: with the workload's eps, then with a
        # threshold that lets about half of the leaves go
        f.upload_interior(un)
        o.set_interior(un)
        eps_half = np.median(det_ref, axis=0) * 8.0
        for e in (eps, eps_half):
            o.sync(cfg.g, cfg.g, ignore_filter=False)
            n_ref = o.adapt(e)
            n = f.adapt(e)
            assert n == n_ref
            a = _sorted(*o.grid(), o.data())
            b = _sorted(*f.grid(), f.download())
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            assert np.array_equal(a[2], b[2])
        assert n < len(lv)


def test_batched_stepper_jmax5_matches_oracle():
    cfg, lv, co, u0, ids, masks = workloads.build("acm3d_sphere_j7", jmax=5)
    assert cfg.rhs_precision == 1 and len(lv) == 3144
    o = Oracle(cfg, threads=16)
    o.set_grid(lv, co, None)
    o.set_interior(u0)
    o.set_mask_sparse(ids, masks)
    t_ref = 0.0
    for _ in range(3):
        t_ref, _ = o.step(t_ref)
    from pyoracle import interior
    ref = interior(cfg, o.data())
    with Context(cfg, len(lv) + 16) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload_interior(u0)
        f.set_mask_sparse(ids, masks)
        f.set_time(0.0)
        f.run(3, use_graph=True)
        t, _ = f.time()
        got = f.download_interior()
    assert abs(t - t_ref) <= 1e-12 * t_ref
    err = float(np.linalg.norm(got - ref.reshape(got.shape)) / np.linalg.norm(ref))
    assert err < 1e-10, err
