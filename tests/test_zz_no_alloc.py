"""The allocation-free coarsening indicator (wg_threshold_flags_noalloc).

It serves callers that may not allocate device memory during a call, such as
a host code that manages its own device memory pool or runs under a device
memory budget enforced outside CUDA: its scratch is a static device array.
This test calls it through the C ABI on device buffers the test allocates,
twice in a row with different inputs, and compares flags and details with the
context-based wg_threshold_flags, which must agree exactly (both evaluate the
same bit-exact kernels).
"""
import ctypes

import numpy as np
import pytest

from helpers import small_cfg, smooth_state
from wabbit_gb300 import capi, grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _call_noalloc(cfg, synced, eps, with_details=True, side_stream=False):
    """One call on device buffers the test owns; returns flags and details
    (None without a details buffer)."""
    L = capi.load()
    nblk = synced.shape[0]
    d_blocks = torch.from_numpy(np.ascontiguousarray(synced)).cuda()
    d_flags = torch.full((nblk,), 7, dtype=torch.int32, device="cuda")
    d_det = torch.full((nblk, cfg.neq), -3.0, dtype=torch.float64, device="cuda") if with_details else None
    eps = np.ascontiguousarray(eps, np.float64)
    torch.cuda.synchronize()
    s = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    capi.check(L.wg_threshold_flags_noalloc(ctypes.byref(cfg), nblk, d_blocks.data_ptr(),
                                            eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            d_flags.data_ptr(), d_det.data_ptr() if with_details else None,
                                            s.cuda_stream))
    s.synchronize()
    return d_flags.cpu().numpy(), (d_det.cpu().numpy() if with_details else None)


@pytest.mark.parametrize("dim,wavelet", [(2, "CDF40"), (3, "CDF44")])
def test_noalloc_flags_match_context_path_twice(dim, wavelet):
    cfg = small_cfg(dim, wavelet, Bs=8 if dim == 2 else 12, jmin=2 if dim == 2 else 1,
                    jmax=4 if dim == 2 else 2)
    lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=17, frac=0.3)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        for call, seed in enumerate((31, 32)):
            f.upload(smooth_state(cfg, lv, co, seed))
            f.sync_ghosts_tree()
            _, det0 = f.coarseningIndicator(np.full(cfg.neq, 1.0))
            eps = np.median(det0, axis=0) * (1.0 + 0.1 * call)
            ref_flags, ref_det = f.coarseningIndicator(eps)
            synced = f.download()
            flags, det = _call_noalloc(cfg, synced, eps)
            assert np.array_equal(flags, ref_flags)
            assert np.array_equal(det, ref_det)
            assert (flags == -1).any() and (flags == 0).any()


@pytest.mark.parametrize("with_details,side_stream", [(False, False), (True, True), (False, True)])
def test_noalloc_without_details_and_on_a_side_stream(with_details, side_stream):
    cfg = small_cfg(2, "CDF40", Bs=8, jmin=2, jmax=4)
    lv, co = grids.random_graded(2, cfg.Jmin, cfg.Jmax, seed=23, frac=0.3)
    with Context(cfg, len(lv) + 4) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(smooth_state(cfg, lv, co, 41))
        f.sync_ghosts_tree()
        _, det0 = f.coarseningIndicator(np.full(cfg.neq, 1.0))
        eps = np.median(det0, axis=0)
        ref_flags, ref_det = f.coarseningIndicator(eps)
        synced = f.download()
    for _ in range(2):
        flags, det = _call_noalloc(cfg, synced, eps, with_details, side_stream)
        assert np.array_equal(flags, ref_flags)
        if with_details:
            assert np.array_equal(det, ref_det)


def test_noalloc_and_context_alternate_wavelets():
    """CDF4,0 and CDF4,4 calls alternate between the allocation-free entry
    and two contexts: each result equals the same call made alone (the
    filters of a launch travel with it, nothing is left behind for the next
    call)."""
    cases = {}
    for w in ("CDF40", "CDF44"):
        cfg = small_cfg(2, w, Bs=12, jmin=2, jmax=4)
        lv, co = grids.random_graded(2, cfg.Jmin, cfg.Jmax, seed=29, frac=0.3)
        ctx = Context(cfg, len(lv) + 4)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(smooth_state(cfg, lv, co, 43))
        f.sync_ghosts_tree()
        _, det0 = f.coarseningIndicator(np.full(cfg.neq, 1.0))
        eps = np.median(det0, axis=0)
        alone = f.coarseningIndicator(eps)
        cases[w] = (cfg, ctx, f, eps, alone, f.download())
    try:
        for rnd in range(3):
            for w in (("CDF40", "CDF44") if rnd % 2 == 0 else ("CDF44", "CDF40")):
                cfg, ctx, f, eps, (ref_flags, ref_det), synced = cases[w]
                flags, det = _call_noalloc(cfg, synced, eps, True, side_stream=rnd == 1)
                assert np.array_equal(flags, ref_flags) and np.array_equal(det, ref_det), w
                other = cases["CDF44" if w == "CDF40" else "CDF40"]
                oflags, odet = other[2].coarseningIndicator(other[3])
                assert np.array_equal(oflags, other[4][0]) and np.array_equal(odet, other[4][1])
    finally:
        for v in cases.values():
            v[1].close()


def test_noalloc_rejects_blocks_too_large_for_one_thread_block():
    cfg = small_cfg(3, "CDF44", Bs=24, jmin=1, jmax=2)
    L = capi.load()
    eps = np.ones(cfg.neq)
    st = L.wg_threshold_flags_noalloc(ctypes.byref(cfg), 4, ctypes.c_void_p(16),
                                      eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      ctypes.c_void_p(16), None, None)
    assert st == -1
    assert b"does not fit" in L.wg_last_error()


def test_noalloc_rejects_too_many_blocks():
    cfg = small_cfg(2, "CDF40", Bs=8, jmin=2, jmax=3)
    L = capi.load()
    eps = np.ones(cfg.neq)
    st = L.wg_threshold_flags_noalloc(ctypes.byref(cfg), 16385, ctypes.c_void_p(16),
                                      eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      ctypes.c_void_p(16), None, None)
    assert st == -1
    assert b"16384" in L.wg_last_error()
