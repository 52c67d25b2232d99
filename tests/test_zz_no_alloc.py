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


def _call_noalloc(cfg, synced, eps):
    L = capi.load()
    nblk = synced.shape[0]
    d_blocks = torch.from_numpy(np.ascontiguousarray(synced)).cuda()
    d_flags = torch.full((nblk,), 7, dtype=torch.int32, device="cuda")
    d_det = torch.full((nblk, cfg.neq), -3.0, dtype=torch.float64, device="cuda")
    eps = np.ascontiguousarray(eps, np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(L.wg_threshold_flags_noalloc(ctypes.byref(cfg), nblk, d_blocks.data_ptr(),
                                            eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            d_flags.data_ptr(), d_det.data_ptr(), stream))
    torch.cuda.synchronize()
    return d_flags.cpu().numpy(), d_det.cpu().numpy()


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


def test_noalloc_rejects_too_many_blocks():
    cfg = small_cfg(2, "CDF40", Bs=8, jmin=2, jmax=3)
    L = capi.load()
    eps = np.ones(cfg.neq)
    st = L.wg_threshold_flags_noalloc(ctypes.byref(cfg), 16385, ctypes.c_void_p(16),
                                      eps.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      ctypes.c_void_p(16), None, None)
    assert st == -1
    assert b"16384" in L.wg_last_error()
