"""The reference's cylinder regression runs (TESTING/acm/acm_CDF40,
acm_CDF44) through the C ABI on the GPU: the tree draws its masks from the
cylinder geometry with the p-norm sponge, normalises eps itself and applies
mask thresholding and max-level dealiasing in wg_adapt, each iteration being
the reference's sync, refine everywhere, RK4 step and adapt_tree
(LIB/MAIN/main.f90:293-427).

* strict variant (no FMA): grid and state bit-identical to the oracle run on
  the same host (the oracle reproduces the reference's CDF4,0 files bit for
  bit, tests/test_acm_cyl.py), and the reference's saved grid;
* fast variant (FMA stencils): the reference's grid, state within 1e-10;
* FP32-pipe precision (double-float stencils, FP64 state): the reference's
  grid, state within relative L2 1e-10 of the oracle;
* the divergence guard (|u| > 1e12, rhs_ACM.f90:133-146) ends the step with
  WG_EDIVERGED in both precisions."""
import os

import numpy as np
import pytest

from acm_cyl_case import Case, reorder, run_library, run_oracle
from helpers import rel_l2
from pyoracle import interior, pad_blocks

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def threads():
    return max(1, min(16, os.cpu_count() or 1))


def oracle_result(case, tend):
    o, it, t = run_oracle(case, tend, threads())
    lv, co = o.grid()
    return (lv, co), interior(case.cfg, o.data()), it, t


@pytest.mark.parametrize("w", ["CDF40", "CDF44"])
def test_cylinder_run_strict_matches_oracle_and_reference_grid(golden, w):
    c = Case(golden, w)
    (glv, gco), u, it, t = run_library(c, 0.05, fast=False)
    (olv, oco), uo, ito, to = oracle_result(c, 0.05)
    assert it == ito == c.iteration("t1") and t == to == 0.05
    perm = reorder(olv, oco, glv, gco)
    assert perm is not None, "library grid differs from the oracle's"
    assert np.array_equal(u[perm], uo), "strict state differs from the oracle"
    perm = reorder(*c.grid("t1"), glv, gco)
    assert perm is not None, "library grid differs from the reference's"
    ref = c.state("t1")
    assert np.abs(u[perm].reshape(ref.shape) - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("w", ["SIG44", "NORM44"])
def test_jmax5_variants_strict_match_oracle_and_reference(golden, w):
    """acm_significant_CDF44 (wg_refine_significant from the status set with
    the t=0 state) and acm_norm_CDF44 (threshold components 2 2 1), 151
    iterations to t=0.2: the strict variant equals the oracle bit for bit
    and ends on the reference's grid."""
    c = Case(golden, w)
    tend = float(c.z["t2_time"])
    (glv, gco), u, it, t = run_library(c, tend, fast=False)
    (olv, oco), uo, ito, to = oracle_result(c, tend)
    assert it == ito == c.iteration("t2") and t == to == tend
    perm = reorder(olv, oco, glv, gco)
    assert perm is not None, "library grid differs from the oracle's"
    assert np.array_equal(u[perm], uo), "strict state differs from the oracle"
    perm = reorder(*c.grid("t2"), glv, gco)
    assert perm is not None, "library grid differs from the reference's"
    ref = c.state("t2")
    assert np.abs(u[perm].reshape(ref.shape) - ref).max() <= 1e-13 * np.abs(ref).max()


def test_cylinder_run_fast_variant(golden):
    c = Case(golden, "CDF40")
    (glv, gco), u, it, _ = run_library(c, 0.05, fast=True)
    assert it == c.iteration("t1")
    perm = reorder(*c.grid("t1"), glv, gco)
    assert perm is not None, "fast-variant grid differs from the reference's"
    ref = c.state("t1")
    assert np.abs(u[perm].reshape(ref.shape) - ref).max() <= 1e-10 * np.abs(ref).max()


def test_cylinder_run_fp32_pipe(golden):
    c = Case(golden, "CDF40")
    (glv, gco), u, it, _ = run_library(c, 0.05, fast=True, precision=1)
    assert it == c.iteration("t1")
    perm = reorder(*c.grid("t1"), glv, gco)
    assert perm is not None, "FP32-pipe grid differs from the reference's"
    ref = c.state("t1")
    assert rel_l2(u[perm].reshape(ref.shape), ref) <= 1e-10


@pytest.mark.parametrize("precision", [0, 1])
def test_divergence_guard(golden, precision):
    from wabbit_gb300 import capi
    from wabbit_gb300.solver import Context

    c = Case(golden, "CDF40")
    cfg = c.cfg.copy()
    cfg.rhs_precision = precision
    lv, co = c.grid("t0")
    u = c.state("t0").copy()
    with Context(cfg, 400) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.set_geometry(c.geo)
        f.upload(pad_blocks(cfg, u))
        f.set_time(0.0)
        f.timeStep_tree()                       # a regular step passes
        u[5, 0, 11, 3] = 1.0e13
        f.upload(pad_blocks(cfg, u))
        f.set_time(0.0)
        with pytest.raises(capi.WgError) as e:
            f.timeStep_tree()
        assert e.value.code == capi.ERRORS_BY_NAME["WG_EDIVERGED"]
        u[5, 0, 11, 3] = -0.5                   # a clean state steps again
        f.upload(pad_blocks(cfg, u))
        f.set_time(0.0)
        f.timeStep_tree()
