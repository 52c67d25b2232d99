"""Interior state transfers through the C ABI: page-locked host buffers are
read and written in place by the copy kernels, pageable ones go through the
staging buffer; both must give the same state."""
import numpy as np
import pytest

from helpers import small_cfg
from wabbit_gb300 import grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


@pytest.mark.parametrize("dim", [2, 3])
def test_interior_roundtrip_pinned_and_pageable(dim):
    cfg = small_cfg(dim, "CDF44" if dim == 3 else "CDF40", Bs=16, jmin=1, jmax=3 if dim == 3 else 4)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=5, frac=0.4)
    rng = np.random.default_rng(3)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        u = rng.standard_normal((len(lv),) + f.interior_shape)
        pin_in = torch.empty(u.shape, dtype=torch.float64, pin_memory=True).numpy()
        pin_in[...] = u
        f.upload_interior(pin_in)
        full_pinned = f.download()
        assert np.array_equal(f.download_interior(), u)
        pin_out = torch.zeros(u.shape, dtype=torch.float64, pin_memory=True).numpy()
        f.download_interior(pin_out)
        assert np.array_equal(pin_out, u)
        f.upload_interior(np.ascontiguousarray(u))
        assert np.array_equal(f.download(), full_pinned)


@pytest.mark.parametrize("precision,scales", [(0, (1, 1, 1, 1)), (1, (1, 1, 1, 1)), (1, (1, 8, 0.25, 3, 3))])
def test_rk4_stream_equals_upload_step_download(precision, scales):
    """wg_rk4_stream (overlapped transfers, five staging buffers; with the
    FP32-pipe precision the last stage of a step loads the next input) gives,
    step by step, the same results as upload + wg_rk4_step + download, also
    when the inputs' magnitudes change the anchoring quantum between steps,
    and leaves the last result as the state."""
    cfg = small_cfg(3, "CDF44", Bs=16, jmin=1, jmax=2)
    cfg.rhs_precision = precision
    lv, co = grids.random_graded(3, cfg.Jmin, cfg.Jmax, seed=7, frac=0.5)
    rng = np.random.default_rng(9)
    nsteps = len(scales)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        shape = (len(lv),) + f.interior_shape
        ins = [torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(nsteps)]
        for a, sc in zip(ins, scales):
            a[...] = 0.1 * sc * rng.standard_normal(shape)
        outs = [torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(nsteps)]
        f.set_time(0.0)
        f.rk4_stream(ins, outs)
        t_stream = f.time()
        assert np.array_equal(f.download_interior(), outs[-1])
        f.timeStep_tree()
        after = f.download_interior()
        f.set_time(0.0)
        for k in range(nsteps):
            f.upload_interior(ins[k])
            f.timeStep_tree()
            ref = f.download_interior()
            assert np.array_equal(outs[k], ref), k
        assert f.time() == t_stream
        f.timeStep_tree()
        assert np.array_equal(f.download_interior(), after)


@pytest.mark.parametrize("dim,penal", [(2, 0), (3, 0), (3, 1)])
def test_dt_from_recorded_maxima_equals_state_scan(dim, penal):
    """FP32-pipe precision: the dt reduction of a step reads the per-block
    maxima of |u|^2 that the previous step's last stage recorded; steps
    replayed from the graph give the same states and times, bit for bit, as
    steps each preceded by wg_compute_dt (which scans the state, so that the
    step's own reduction scans it too)."""
    cfg = small_cfg(dim, "CDF44" if dim == 3 else "CDF40", Bs=16, jmin=1, jmax=2 if dim == 3 else 3, penal=penal)
    cfg.rhs_precision = 1
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=11, frac=0.5)
    rng = np.random.default_rng(12)
    shape = (len(lv), cfg.neq, cfg.Bs[2] if dim == 3 else 1, cfg.Bs[1], cfg.Bs[0])
    u0 = 0.2 * rng.standard_normal(shape)
    nsteps = 6
    res = []
    for scan in (False, True):
        with Context(cfg, len(lv) + 4) as ctx:
            f = ctx.forest()
            f.set_grid(lv, co)
            if penal:
                f.set_mask_sphere((0.5, 0.6, 0.7), 0.3)
            f.upload_interior(u0)
            f.set_time(0.0)
            if scan:
                for _ in range(nsteps):
                    f.calculate_time_step()
                    f.timeStep_tree()
            else:
                f.run(nsteps, use_graph=True)
            res.append((f.download_interior(), f.time()))
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1]


def test_stream_divergence_guard_on_the_next_input():
    """FP32-pipe stream: the divergence guard of a step's input is taken by
    the previous step's last stage, which loads it; an input with a value
    above 1e12 makes the tree report WG_EDIVERGED, as the same input uploaded
    does."""
    from wabbit_gb300 import capi

    cfg = small_cfg(3, "CDF44", Bs=16, jmin=1, jmax=2)
    cfg.rhs_precision = 1
    lv, co = grids.random_graded(3, cfg.Jmin, cfg.Jmax, seed=7, frac=0.5)
    rng = np.random.default_rng(13)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        shape = (len(lv),) + f.interior_shape
        ins = [torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
        for a in ins:
            a[...] = 0.1 * rng.standard_normal(shape)
        outs = [torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
        f.set_time(0.0)
        f.rk4_stream(ins, outs)
        f.time()                                  # clean inputs: no flag
        ins[1][2, 3, 5, 4, 1] = 1.0e13
        f.set_time(0.0)
        f.rk4_stream(ins, outs)
        with pytest.raises(capi.WgError) as e:
            f.time()
        assert e.value.code == capi.ERRORS_BY_NAME["WG_EDIVERGED"]
        f.upload_interior(ins[1])
        f.set_time(0.0)
        with pytest.raises(capi.WgError) as e:
            f.timeStep_tree()
        assert e.value.code == capi.ERRORS_BY_NAME["WG_EDIVERGED"]
