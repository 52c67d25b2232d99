"""The oracle against the reference's adaptive 2-D ACM runs
TESTING/acm/3vortices/3vorticesAdaptFD4_CDF40 and _CDF42 (PARAMS_3vortices.ini):
skew-symmetric FD4, CDF4,0 or CDF4,2 with coarse extension and security zone
(useCoarseExtension=1, useSecurityZone=1), threshold-state-vector coarsening
with eps normalised by the Linfty norm, refinement "significant" (the blocks
the previous adaptation found significant), one RK4 step per grid. The
reference's main loop (LIB/MAIN/main.f90:293-427): the state read at t=10 is
adapted once (adapt_inicond, setInitialCondition_tree.f90:80-84), then every
iteration runs sync_ghosts_tree, refine_tree(significant), timeStep_tree and
adapt_tree until t=15."""
import os

import numpy as np
import pytest

from acm_cyl_case import reorder
from pyoracle import Oracle, interior, pad_blocks
from wabbit_gb300 import config


def load_case(golden, wavelet="CDF40"):
    """The fixture entries of one of the two cases (CDF4,0 unprefixed)."""
    z0 = golden("vortex2d_adapt.npz")
    pre = "" if wavelet == "CDF40" else wavelet + "_"
    return {k[len(pre):]: z0[k] for k in z0.files if k.startswith(pre) and (pre or not k.startswith("CDF"))}


def _case(golden, wavelet="CDF40"):
    z = load_case(golden, wavelet)
    cfg = config.from_ini_text(str(z["ini"]))
    o = Oracle(cfg, threads=os.cpu_count() or 1)
    o.set_coarse_extension(True)
    o.set_grid(z["t10_level"], z["t10_coords"], pad_blocks(cfg, z["t10_u"]))
    return z, cfg, o


def _iteration(cfg, o, t):
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    nref = o.refine_significant()
    t, _ = o.step(t)
    o.adapt(o.eps_use())
    return t, nref


def test_ini_of_the_adaptive_case(golden):
    z, cfg, _ = _case(golden)
    assert cfg.dim == 2 and list(cfg.Bs[:2]) == [32, 32] and cfg.skew_symmetry == 1
    assert bytes(cfg.wavelet).rstrip(b"\0").decode() == "CDF40"
    assert (cfg.Jmin, cfg.Jmax, cfg.eps, cfg.eps_normalized) == (1, 4, 1e-3, 1)


def test_significant_refinement_first_iterations(golden):
    """The status an adaptation leaves is 0 (significant) or
    REF_UNSIGNIFICANT_STAY (9); the significant blocks refine, the others
    only where gradedness asks for it, so the refined grid has fewer blocks
    than refinement everywhere would give, and it stays graded."""
    z, cfg, o = _case(golden)
    o.adapt(o.eps_use())
    t = float(z["t10_time"])
    for _ in range(3):
        st = o.status()
        assert set(np.unique(st)) <= {0, 9} and (st == 0).any()
        lv, _ = o.grid()
        everywhere = int(np.sum(np.where(lv < cfg.Jmax, 4, 1)))
        t, nref = _iteration(cfg, o, t)
        assert len(lv) < nref < everywhere


@pytest.mark.slow
@pytest.mark.parametrize("wavelet", ["CDF40"])
def test_adaptive_run_t10_to_t15_matches_reference(golden, wavelet):
    """2281 adaptive iterations t=10 -> 15 (the reference's iteration count)
    end on the reference's grid (61 blocks on levels 2-4); the values agree
    to 1e-13 of the field maximum (observed 8e-15: the coarse-extension
    reconstruction of the reference is not reproduced bit for bit, as for
    the CDF4,4 runs). The CDF4,2 case (58 blocks, 1.1e-14) takes two minutes
    on 16 cores in the oracle; its run to t=15 is checked through the device
    path, which equals the oracle bit for bit in its strict variant
    (test_gpu_vortex2d_adapt.py)."""
    z, cfg, o = _case(golden, wavelet)
    o.adapt(o.eps_use())
    t, it = float(z["t10_time"]), 0
    while t < float(z["t15_time"]) - 1e-12:
        t, _ = _iteration(cfg, o, t)
        it += 1
    assert it == int(z["t15_iteration"] - z["t10_iteration"]) and t == float(z["t15_time"])
    lv, co = o.grid()
    perm = reorder(z["t15_level"], z["t15_coords"], lv, co)
    assert perm is not None, "adapted grid differs from the reference's"
    u = interior(cfg, o.data())[perm].reshape(z["t15_u"].shape)
    assert np.abs(u - z["t15_u"]).max() <= 1e-13 * np.abs(z["t15_u"]).max()
