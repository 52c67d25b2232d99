"""Penalisation mask of a fixed sphere computed on the device
(wg_set_mask_sphere; create_mask_3D_acm 'sphere-fixed' -> draw_sphere,
LIB/EQUATION/ACMnew/create_mask.f90:58-61,
LIB/EQUATION/insects/module_geometry.f90:49-117) against the host mask of the
workloads: the same blocks carry a mask, colour / u_s / sponge are equal and
chi agrees to the last bits (only the cosine of the smoothing zone may differ
by an ulp); an RK4 step with either mask gives the same state within 1e-12."""
import numpy as np
import pytest

from helpers import small_cfg, smooth_state
from wabbit_gb300 import grids, workloads
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


@pytest.mark.parametrize("precision", [0, 1])
def test_sphere_mask_on_device_matches_host(precision):
    cfg = small_cfg(3, "CDF40", Bs=16, jmin=2, jmax=4, penal=1)
    cfg.C_eta = 1e-3
    cfg.rhs_precision = precision
    centre = [0.5 * cfg.domain[d] for d in range(3)]
    radius = 0.2
    lv, co = grids.refined_around(3, cfg.Jmin, cfg.Jmax, list(cfg.domain), centre, lambda level: radius + 0.1)
    ids, masks = workloads.sphere_mask(cfg, lv, co, centre=centre, radius=radius, C_smooth=1.5)
    assert len(ids) > 0
    data = smooth_state(cfg, lv, co, 3)
    with Context(cfg, 2 * len(lv) + 8) as ctx:
        ctx.set_variant(False)
        fh = ctx.forest()
        fh.set_grid(lv, co)
        fh.upload(data)
        fh.set_mask_sparse(ids, masks)
        fd = ctx.forest()
        fd.set_grid(lv, co)
        fd.upload(data)
        fd.set_mask_sphere(centre, radius, 1.5)
        assert fh.stats()[1] == fd.stats()[1] > 0
        worst = 0.0
        for b in range(len(lv)):
            mh, md = fh.mask_block(b), fd.mask_block(b)
            assert (mh is None) == (md is None), b
            if mh is None:
                continue
            assert np.array_equal(mh[1:], md[1:]), b
            worst = max(worst, float(np.abs(mh[0] - md[0]).max()))
        assert worst <= 1e-15
        for f in (fh, fd):
            f.set_time(0.0)
            f.timeStep_tree()
        a, b2 = fh.download(), fd.download()
    assert np.abs(a - b2).max() <= 1e-12 * np.abs(a).max()
