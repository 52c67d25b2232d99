"""The library on the reference's adaptive 2-D ACM runs
TESTING/acm/3vortices/3vorticesAdaptFD4_CDF40 and _CDF42: CDF4,0 with the
coarse extension and security zone its ini switches on
(use_coarse_extension), or the lifted CDF4,2,
refinement "significant" (wg_refine_significant on the status the last
wg_adapt left), one RK4 step per grid, the main loop of
LIB/MAIN/main.f90:293-427 after the adaptation of the state read at t=10.
The strict variant is compared with the oracle bit for bit, the run to
t=15 with the reference's saved state."""
import numpy as np
import pytest

from acm_cyl_case import reorder
from pyoracle import Oracle, interior, pad_blocks
from test_vortex2d_adapt import load_case
from wabbit_gb300 import config

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _cfg(z):
    cfg = config.from_ini_text(str(z["ini"]))
    assert cfg.use_coarse_extension == 1
    return cfg


def _run_library(z, cfg, nit=None, fast=False):
    from wabbit_gb300.solver import Context
    with Context(cfg, 1200) as ctx:
        ctx.set_variant(fast)
        f = ctx.forest()
        f.set_grid(z["t10_level"], z["t10_coords"])
        f.upload(pad_blocks(cfg, z["t10_u"]))
        t = float(z["t10_time"])
        f.set_time(t)
        f.adapt()
        status0 = f.refinement_status()
        it = 0
        while t < float(z["t15_time"]) - 1e-12 and (nit is None or it < nit):
            f.sync_ghosts_tree()
            f.refine_significant()
            t, _ = f.timeStep_tree()
            f.adapt()
            it += 1
        lv, co = f.grid()
        return (lv, co), interior(cfg, f.download()), it, t, status0


def _run_oracle(z, cfg, nit):
    o = Oracle(cfg)
    o.set_grid(z["t10_level"], z["t10_coords"], pad_blocks(cfg, z["t10_u"]))
    t = float(z["t10_time"])
    o.adapt(o.eps_use())
    status0 = o.status()
    for _ in range(nit):
        o.sync(cfg.g, cfg.g, ignore_filter=True)
        o.refine_significant()
        t, _ = o.step(t)
        o.adapt(o.eps_use())
    return o.grid(), interior(cfg, o.data()), t, status0


@pytest.mark.parametrize("wavelet", ["CDF40", "CDF42"])
def test_adaptive_loop_strict_matches_oracle(golden, wavelet):
    """40 iterations: the same refinement status after the first
    adaptation, the same grids and bit-identical states and times."""
    z = load_case(golden, wavelet)
    cfg = _cfg(z)
    (glv, gco), u, it, t, s0 = _run_library(z, cfg, nit=40)
    (olv, oco), uo, to, so = _run_oracle(z, cfg, 40)
    assert it == 40 and t == to
    assert np.array_equal(np.sort(s0), np.sort(so)) and set(np.unique(s0)) <= {0, 9}
    perm = reorder(olv, oco, glv, gco)
    assert perm is not None, "library grid differs from the oracle's"
    assert np.array_equal(u[perm], uo)


def test_refine_significant_needs_a_status(golden):
    from wabbit_gb300 import capi
    from wabbit_gb300.solver import Context
    z = load_case(golden)
    cfg = _cfg(z)
    with Context(cfg, 200) as ctx:
        f = ctx.forest()
        f.set_grid(z["t10_level"], z["t10_coords"])
        with pytest.raises(capi.WgError):
            f.refine_significant()


@pytest.mark.slow
@pytest.mark.parametrize("wavelet", ["CDF40", "CDF42"])
def test_adaptive_run_t10_to_t15_matches_reference(golden, wavelet):
    """The reference's 2281 iterations end on its grid (61 / 58 blocks);
    the values agree to 1e-13 of the field maximum (the oracle's own
    agreement)."""
    z = load_case(golden, wavelet)
    cfg = _cfg(z)
    (glv, gco), u, it, t, _ = _run_library(z, cfg)
    assert it == int(z["t15_iteration"] - z["t10_iteration"]) and t == float(z["t15_time"])
    perm = reorder(z["t15_level"], z["t15_coords"], glv, gco)
    assert perm is not None, "adapted grid differs from the reference's"
    ref = z["t15_u"]
    assert np.abs(u[perm].reshape(ref.shape) - ref).max() <= 1e-13 * np.abs(ref).max()
