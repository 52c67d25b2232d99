"""GPU hot path against the CPU oracle and the reference's regression files.

Bit-exactness bar: the sync, the dt, the strict-variant RHS/RK4 and the
wavelet details are computed with the reference's rounding and must match
bit for bit. The fast (FMA) variant must agree within relative L2 <= 1e-12
per step (spec tolerance), and within 1e-10 after thousands of steps.
"""
import numpy as np
import pytest

from helpers import rel_l2, random_state, small_cfg, smooth_state, sphere_mask, vortex_cfg
from pyoracle import Oracle, interior, pad_blocks
from wabbit_gb300 import config, grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


@pytest.fixture(scope="module")
def grids2d():
    return grids.random_graded(2, 2, 5, seed=11, frac=0.3)


@pytest.fixture(scope="module")
def grids3d():
    return grids.random_graded(3, 1, 3, seed=5, frac=0.3)


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (3, "CDF40"), (2, "CDF20"), (2, "CDF60")])
@pytest.mark.parametrize("full", [False, True])
def test_sync_bitexact(dim, wavelet, full, grids2d, grids3d):
    g, _ = config.wavelet_ghosts(wavelet)
    cfg = small_cfg(dim, wavelet, Bs=8 if 2 * g - 1 <= 8 else 16, jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    lv, co = grids2d if dim == 2 else grids3d
    data = random_state(cfg, len(lv), 3)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    gm = cfg.g if full else cfg.g_rhs
    o.sync(gm, gm, ignore_filter=True)
    with Context(cfg, len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        if full:
            f.sync_ghosts_tree()
        else:
            f.sync_ghosts_RHS_tree()
        got = f.download()
    assert np.array_equal(got, o.data())


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("skew", [0, 1])
def test_rhs_strict_bitexact_fast_close(dim, skew, grids2d, grids3d):
    cfg = small_cfg(dim, skew=skew, jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    lv, co = grids2d if dim == 2 else grids3d
    data = smooth_state(cfg, lv, co, 7)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.sync()
    ref = interior(cfg, o.rhs())
    with Context(cfg, len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.sync_ghosts_RHS_tree()
        ctx.set_variant(False)
        strict = interior(cfg, f.RHS_ACM())
        ctx.set_variant(True)
        fast = interior(cfg, f.RHS_ACM())
    assert np.array_equal(strict, ref)
    assert rel_l2(fast, ref) < 1e-12


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("penal", [0, 1])
def test_rk4_steps_strict_bitexact(dim, penal, grids2d, grids3d):
    cfg = small_cfg(dim, skew=0, penal=penal, jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    cfg.C_eta = 1e-2
    lv, co = grids2d if dim == 2 else grids3d
    data = smooth_state(cfg, lv, co, 9)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.2) if penal else None
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.set_mask(mask)
    with Context(cfg, len(lv) + 8) as ctx:
        ctx.set_variant(False)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_mask(mask)
        f.set_time(0.0)
        t_ref = 0.0
        for _ in range(3):
            t_ref, dt_ref = o.step(t_ref)
            t, dt = f.timeStep_tree()
            assert dt == dt_ref and t == t_ref
        got = interior(cfg, f.download())
    assert np.array_equal(got, interior(cfg, o.data()))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("skew,penal", [(1, 0), (0, 0), (0, 1)])
def test_rk4_fast_within_tolerance(dim, skew, penal, grids2d, grids3d):
    """Fast variant (regrouped FMA stencils): relative L2 <= 1e-12 per step."""
    cfg = small_cfg(dim, skew=skew, penal=penal, jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    cfg.C_eta = 1e-2
    lv, co = grids2d if dim == 2 else grids3d
    data = smooth_state(cfg, lv, co, 13)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.2) if penal else None
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.set_mask(mask)
    with Context(cfg, len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_mask(mask)
        f.set_time(0.0)
        t_ref = 0.0
        for _ in range(5):
            t_ref, _ = o.step(t_ref)
            f.timeStep_tree()
            err = rel_l2(interior(cfg, f.download()), interior(cfg, o.data()))
            assert err < 1e-12


@pytest.mark.parametrize("fast", [False, True])
def test_vortex2d_reference_golden(golden, fast):
    """3073 RK4 steps of the reference's 3vorticesEquiFD4_CDF40 case on the GPU."""
    z = golden("vortex2d_equi.npz")
    cfg = vortex_cfg()
    nsteps = len(z["log_time"])
    with Context(cfg, 80) as ctx:
        ctx.set_variant(fast)
        f = ctx.forest()
        f.set_grid(z["level"], z["coords"])
        f.upload(pad_blocks(cfg, z["u_in"]))
        f.set_time(float(z["t_in"]))
        f.run(nsteps, use_graph=True)
        t, dt = f.time()
        u = interior(cfg, f.download())
    assert t == 20.0
    if fast:
        assert rel_l2(u, z["u_out"]) < 1e-10
    else:
        assert np.array_equal(u, z["u_out"])


def test_tg3d_reference_golden(golden):
    z = golden("tg3d_equi.npz")
    c = config.defaults(3)
    c.Bs[:] = (20, 20, 20)
    c.domain[:] = (6.283185307179586,) * 3
    c.g, c.g_rhs = 3, 2
    c.Jmin = c.Jmax = 1
    c.c0, c.nu, c.gamma_p = 10.0, 3.125e-03, 0.0
    c.skew_symmetry, c.penalization = 1, 0
    c.CFL = 1.0
    c.time_max, c.write_time, c.tsave_stats = 10.0, 10.0, 0.2
    with Context(c, 8) as ctx:
        ctx.set_variant(False)
        f = ctx.forest()
        f.set_grid(z["level"], z["coords"])
        f.upload(pad_blocks(c, z["u_in"]))
        f.set_time(0.0)
        f.run(int(z["iteration_out"]), use_graph=False)
        t, _ = f.time()
        u = interior(c, f.download())
    assert t == 10.0
    assert np.array_equal(u, z["u_out"])


@pytest.mark.parametrize("w", ["CDF40", "CDF20", "CDF60"])
def test_refine_everywhere_reference_golden(golden, w):
    """refineBlock with the order-4, order-2 and order-6 predictors against
    TESTING/wavelets/adaptive_<w>/vor_00100.h5, bit for bit."""
    z = golden("wavelet_adaptive.npz")
    c = config.defaults(2)
    c.Bs[0] = c.Bs[1] = 32
    c.domain[0] = c.domain[1] = 6.283185307179586
    c.neq = 3  # the context needs dim+1 components: the field goes in component 0
    c.wavelet = w.encode()
    c.g, c.g_rhs = max(3, config.wavelet_ghosts(w)[0]), 2
    c.Jmin, c.Jmax = 1, 7
    key = "refined" if w == "CDF40" else f"refined_{w}"
    u = np.zeros((len(z["in_level"]), 3) + z["in_u"].shape[2:])
    u[:, 0] = z["in_u"][:, 0]
    with Context(c, 600) as ctx:
        f = ctx.forest()
        f.set_grid(z["in_level"], z["in_coords"])
        f.upload(pad_blocks(c, u))
        f.sync_ghosts_tree()
        f.refine_everywhere()
        lv, co = f.grid()
        got = interior(c, f.download())[:, :1]
    order = np.lexsort((co[:, 0], co[:, 1], co[:, 2], lv))
    assert np.array_equal(lv[order], z[f"{key}_level"])
    assert np.array_equal(co[order], z[f"{key}_coords"])
    assert np.array_equal(got[order], z[f"{key}_u"])


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (3, "CDF40"), (2, "CDF44"), (3, "CDF44"), (2, "CDF22")])
def test_threshold_flags_bitexact(dim, wavelet, grids2d, grids3d):
    g, _ = config.wavelet_ghosts(wavelet)
    cfg = small_cfg(dim, wavelet, Bs=8 if 2 * g - 1 <= 8 else 12, jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    lv, co = grids2d if dim == 2 else grids3d
    data = smooth_state(cfg, lv, co, 21)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.sync(cfg.g, cfg.g, ignore_filter=True)
    full = o.data()
    # thresholds near the median detail so both decisions occur
    _, det0 = o.flags(np.full(cfg.neq, 1.0))
    eps = np.median(det0, axis=0)
    fl_ref, det_ref = o.flags(eps)
    with Context(cfg, len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(full)
        fl, det = f.coarseningIndicator(eps)
    assert np.array_equal(det, det_ref)
    assert np.array_equal(fl, fl_ref)
    assert (fl == -1).any() and (fl == 0).any()


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (3, "CDF40"), (2, "CDF44"), (3, "CDF44")])
@pytest.mark.parametrize("penal", [0, 1])
def test_rk4_fp32_pipe_path_within_tolerance(dim, wavelet, penal, grids2d, grids3d):
    """Double-float stencils, stage arithmetic, ghost prediction and
    penalisation on the FP32 units, FP64 state: the relative L2 difference to
    the FP64 oracle grows by at most 3e-13 per step (the anchored stage
    inputs carry about 2^-44 of the state's largest magnitude). The ghost nodes go through the pushed same-level
    copies and the restriction / prediction stages (CDF40: two sync stages,
    CDF44: three)."""
    cfg = small_cfg(dim, wavelet, Bs=8 if wavelet == "CDF40" else 12, skew=0, penal=penal,
                    jmin=1 if dim == 3 else 2, jmax=3 if dim == 3 else 5)
    cfg.C_eta = 1e-2
    cfg.rhs_precision = 1
    lv, co = grids2d if dim == 2 else grids3d
    data = smooth_state(cfg, lv, co, 23)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.2) if penal else None
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.set_mask(mask)
    with Context(cfg, len(lv) + 8) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_mask(mask)
        f.set_time(0.0)
        t_ref = 0.0
        for step in range(6):
            t_ref, dt_ref = o.step(t_ref)
            if step < 3:
                t, dt = f.timeStep_tree()
            else:
                f.run(1, use_graph=True)
                t, dt = f.time()
            # the first dt comes from identical states; later ones from states
            # that differ by rounding, so they may differ in the last bits
            assert dt == dt_ref if step == 0 else abs(dt - dt_ref) <= 1e-12 * dt_ref
            err = rel_l2(interior(cfg, f.download()), interior(cfg, o.data()))
            assert err < 3e-13 * (step + 1), (step, err)


def test_fp32_pipe_stage_forms_bit_identical():
    """The direct, tile, march and pipe forms of the FP32-pipe stage kernel
    do the same arithmetic in the same order: three steps with any per-stage
    mix of forms give the same bits, so the autotuner's choices never change
    a result."""
    cfg = small_cfg(3, "CDF40", Bs=16, penal=1, jmin=1, jmax=2)
    cfg.C_eta = 1e-2
    cfg.rhs_precision = 1
    lv, co = grids.random_graded(3, 1, 2, seed=5, frac=0.4)
    data = smooth_state(cfg, lv, co, 31)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.3)
    out = []
    for forms in (["direct"] * 4, ["tile"] * 4, ["march"] * 4, ["pipe"] * 4, ["tile2"] * 4, ["tile8"] * 4,
                  ["march", "tile", "direct", "march"], ["pipe", "direct", "tile", "pipe"],
                  ["tile2", "tile8", "pipe", "tile8"]):
        with Context(cfg, len(lv) + 4) as ctx:
            ctx.set_stage_forms(forms)
            f = ctx.forest()
            f.set_grid(lv, co)
            f.upload(data)
            f.set_mask(mask)
            f.set_time(0.0)
            f.run(3, use_graph=True)
            assert ctx.stage_forms() == forms
            out.append((forms, f.download(), f.time()))
    for forms, u, t in out[1:]:
        assert t == out[0][2], forms
        assert np.array_equal(u, out[0][1]), forms


def test_fp32_pipe_rejects_skew_symmetric():
    from wabbit_gb300 import capi
    cfg = small_cfg(2, skew=1)
    cfg.rhs_precision = 1
    with pytest.raises(capi.WgError):
        Context(cfg, 8)


@pytest.mark.parametrize("form", ["direct", "tile", "march", "pipe", "tile2", "tile8", "auto"])
def test_fp32_pipe_stage_forms_16cubed(form):
    """3-D 16^3 blocks (the benchmark geometry): the direct-load stage
    kernel, the TMA-staged slab, plane-ring and persistent slab kernels, and the autotuner's
    per-stage picks, all stay within 1e-12 of the FP64 oracle over three
    steps on a graded two-level grid with a masked sphere."""
    cfg = small_cfg(3, "CDF40", Bs=16, penal=1, jmin=1, jmax=2)
    cfg.C_eta = 1e-2
    cfg.rhs_precision = 1
    lv, co = grids.random_graded(3, 1, 2, seed=3, frac=0.4)
    data = smooth_state(cfg, lv, co, 29)
    mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.3)
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.set_mask(mask)
    with Context(cfg, len(lv) + 4) as ctx:
        ctx.set_stage_form(form)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_mask(mask)
        f.set_time(0.0)
        t_ref = 0.0
        for step in range(3):
            t_ref, dt_ref = o.step(t_ref)
            if step == 0:
                f.timeStep_tree()
            else:
                f.run(1, use_graph=True)
            err = rel_l2(interior(cfg, f.download()), interior(cfg, o.data()))
            assert err < 1e-12, (form, step, err)
        forms = ctx.stage_forms()
        assert len(forms) == 4
        assert all(x in (("direct", "tile", "march", "pipe", "tile2", "tile8") if form == "auto" else (form,))
                   for x in forms)
        assert ctx.stage_form() == forms[1]
