"""The oracle against the reference's cylinder regression runs
(TESTING/acm/acm_CDF40, acm_CDF44): convective FD_4th_central, cylinder
penalisation with cosine smoothing, p-norm sponge, eps normalised by the
Linfty norm, mask thresholding and max-level dealiasing, adaptation every
iteration. These pin the arithmetic of the penalised convective RHS, the
sponge and the adaptive loop to the reference's own output."""
import os

import numpy as np
import pytest

from acm_cyl_case import Case, reorder, run_oracle
from pyoracle import Oracle, interior


def threads():
    return max(1, min(8, os.cpu_count() or 1))


@pytest.mark.parametrize("w", ["CDF40", "CDF44"])
def test_ini_of_the_cylinder_case(golden, w):
    c = Case(golden, w)
    cfg, geo = c.cfg, c.geo
    assert (cfg.dim, cfg.Bs[0], cfg.Jmin, cfg.Jmax, cfg.g_rhs) == (2, 26, 1, 6, 2)
    assert cfg.g == (3 if w == "CDF40" else 6)
    assert (cfg.threshold_mask, cfg.force_maxlevel_dealiasing, cfg.eps_normalized) == (1, 1, 1)
    assert (cfg.skew_symmetry, cfg.penalization, cfg.use_sponge) == (0, 1, 1)
    assert (geo.kind, geo.sponge_type, geo.R_cyl, geo.L_sponge, geo.p_sponge) == (1, 1, 0.5, 2.0, 8.0)


@pytest.mark.parametrize("w", ["CDF40", "CDF44"])
@pytest.mark.parametrize("key", ["t0", "t1", "t2"])
def test_mask_matches_reference_files(golden, w, key):
    """createMask_tree's chi (draw_circle with the cosine step) equals the
    reference's saved mask on each saved grid, bit for bit."""
    c = Case(golden, w)
    lv, co = c.grid(key)
    o = Oracle(c.cfg)
    o.set_grid(lv, co, np.zeros((len(lv),) + o.block_shape))
    o.set_geometry(c.geo)
    o.make_mask()
    chi = interior(c.cfg, o.mask())[:, 0]
    assert np.array_equal(chi, c.chi(key).reshape(chi.shape))
    # the sponge reaches the boundary blocks and stays off the centre
    spo = interior(c.cfg, o.mask())[:, 5]
    assert spo.max() == 1.0 and spo.min() == 0.0


def test_cdf40_run_bit_exact(golden):
    """39 adaptive iterations to t=0.05 and 80 to t=0.1 reproduce the
    reference's grids and states bit for bit."""
    c = Case(golden, "CDF40")
    for key in ["t1", "t2"]:
        o, it, t = run_oracle(c, c.z[f"{key}_time"], threads())
        assert it == c.iteration(key) and t == c.z[f"{key}_time"]
        lv, co = o.grid()
        perm = reorder(*c.grid(key), lv, co)
        assert perm is not None, "adapted grid differs from the reference's"
        u = interior(c.cfg, o.data())[perm].reshape(c.state(key).shape)
        assert np.array_equal(u, c.state(key))


def test_cdf44_run_matches_reference(golden):
    """Lifted wavelet (coarse extension, security zone): 40 iterations to
    t=0.05 give the reference's grid; the values agree to 1e-13 (the
    reference's CDF4,4 transform sums are not reproducible bit for bit, see
    the coarsen-everywhere pin)."""
    c = Case(golden, "CDF44")
    o, it, t = run_oracle(c, 0.05, threads())
    assert it == c.iteration("t1")
    lv, co = o.grid()
    perm = reorder(*c.grid("t1"), lv, co)
    assert perm is not None, "adapted grid differs from the reference's"
    u = interior(c.cfg, o.data())[perm].reshape(c.state("t1").shape)
    ref = c.state("t1")
    assert np.abs(u - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("w", ["SIG44", "NORM44"])
def test_jmax5_variants_match_reference(golden, w):
    """The reference's Jmax=5 cylinder variants with CDF4,4, 151 iterations
    to t=0.2: acm_significant_CDF44 (refinement "significant" from the
    status saved with the t=0 state) and acm_norm_CDF44 (threshold
    components 2 2 1: the velocity components share one detail, their
    maximum). Grid identical (112 blocks), values within 1e-13 of the
    maximum (observed 2.6e-14, as for the other CDF4,4 runs)."""
    c = Case(golden, w)
    assert c.significant == (w == "SIG44")
    o, it, t = run_oracle(c, float(c.z["t2_time"]), threads())
    assert it == c.iteration("t2") and t == float(c.z["t2_time"])
    lv, co = o.grid()
    perm = reorder(*c.grid("t2"), lv, co)
    assert perm is not None, "adapted grid differs from the reference's"
    u = interior(c.cfg, o.data())[perm].reshape(c.state("t2").shape)
    ref = c.state("t2")
    assert np.abs(u - ref).max() <= 1e-13 * np.abs(ref).max()
    if c.significant:
        assert np.array_equal(np.sort(o.status()), np.sort(c.status("t2")))


def test_divergence_guard_in_oracle(golden):
    """|u| > 1e12 anywhere stops the RHS (rhs_ACM.f90:133-146)."""
    from pyoracle import pad_blocks

    c = Case(golden, "CDF40")
    lv, co = c.grid("t0")
    u = c.state("t0").copy()
    u[3, 1, 7, 9] = 1.0e13
    o = Oracle(c.cfg)
    o.set_grid(lv, co, pad_blocks(c.cfg, u))
    o.set_geometry(c.geo)
    o.make_mask()
    with pytest.raises(RuntimeError, match="-4"):
        o.step(0.0)
