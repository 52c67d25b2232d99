"""ctypes binding of libwabbit_gb300.so (include/wabbit_gb300.h).

There is no CPU fallback: if the library has not been built, or no CUDA
device is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

from .config import WgConfig, WgGeometry

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libwabbit_gb300.so")

WG_OK = 0
ERRORS = {-1: "WG_EINVAL", -2: "WG_ENOMEM", -3: "WG_ECUDA", -4: "WG_EDIVERGED", -5: "WG_ETIMEOUT",
          -6: "WG_EGRID", -7: "WG_ENOTSUP"}
ERRORS_BY_NAME = {v: k for k, v in ERRORS.items()}

# every symbol the header declares (checked by the CPU tests)
EXPORTS = [
    "wg_config_defaults", "wg_last_error", "wg_bytes_per_block", "wg_ctx_create", "wg_ctx_destroy",
    "wg_set_variant", "wg_synchronize", "wg_stream", "wg_tree_create", "wg_tree_destroy", "wg_set_grid",
    "wg_get_nblocks", "wg_get_grid", "wg_upload_state", "wg_download_state", "wg_set_mask", "wg_set_time",
    "wg_get_time", "wg_sync_ghosts", "wg_rhs", "wg_compute_dt", "wg_rk4_step", "wg_run", "wg_threshold_flags",
    "wg_refine_everywhere", "wg_sync_table", "wg_block_slot", "wg_sync_table_host",
    "wg_time_kernel", "wg_tree_stats", "wg_set_mask_sparse", "wg_set_mask_sphere",
    "wg_get_mask_block",
    "wg_upload_interior", "wg_download_interior", "wg_graph_kernels",
    "wg_threshold_flags_noalloc", "wg_set_stage_form", "wg_get_stage_form",
    "wg_wavelet_decompose", "wg_wavelet_reconstruct", "wg_wavelet_threshold", "wg_threshold_flags_wd",
    "wg_adapt", "wg_adapt_profile", "wg_rk4_stream", "wg_set_geometry", "wg_get_stage_forms",
    "wg_step_profile", "wg_set_stage_forms", "wg_refine_significant", "wg_get_refinement_status",
    "wg_set_refinement_status",
]


class WgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_i = ctypes.c_int

_SIGS = {
    "wg_config_defaults": (_i, [ctypes.POINTER(WgConfig), _i]),
    "wg_last_error": (ctypes.c_char_p, []),
    "wg_bytes_per_block": (ctypes.c_size_t, [ctypes.POINTER(WgConfig)]),
    "wg_ctx_create": (_i, [ctypes.POINTER(WgConfig), _i, ctypes.POINTER(_vp)]),
    "wg_ctx_destroy": (_i, [_vp]),
    "wg_set_variant": (_i, [_vp, _i]),
    "wg_set_stage_form": (_i, [_vp, _i]),
    "wg_wavelet_decompose": (_i, [_vp, _i]),
    "wg_adapt": (_i, [_vp, _i, _dp, _i, ctypes.POINTER(ctypes.c_int)]),
    "wg_adapt_profile": (_i, [_vp, _i, _dp, _i]),
    "wg_rk4_stream": (_i, [_vp, _i, _i, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "wg_wavelet_reconstruct": (_i, [_vp, _i]),
    "wg_wavelet_threshold": (_i, [_vp, _i, _dp]),
    "wg_get_stage_form": (_i, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "wg_get_stage_forms": (_i, [_vp, _ip]),
    "wg_step_profile": (_i, [_vp, _i, _ip, _i, _dp]),
    "wg_set_stage_forms": (_i, [_vp, _ip]),
    "wg_synchronize": (_i, [_vp]),
    "wg_stream": (_vp, [_vp]),
    "wg_tree_create": (_i, [_vp, ctypes.POINTER(WgConfig), _ip]),
    "wg_tree_destroy": (_i, [_vp, _i]),
    "wg_set_grid": (_i, [_vp, _i, _i, _ip, _ip]),
    "wg_get_nblocks": (_i, [_vp, _i, _ip]),
    "wg_get_grid": (_i, [_vp, _i, _i, _ip, _ip]),
    "wg_upload_state": (_i, [_vp, _i, _dp]),
    "wg_download_state": (_i, [_vp, _i, _dp]),
    "wg_set_mask": (_i, [_vp, _i, _dp]),
    "wg_set_time": (_i, [_vp, _i, ctypes.c_double]),
    "wg_get_time": (_i, [_vp, _i, _dp, _dp]),
    "wg_sync_ghosts": (_i, [_vp, _i, _i, _i]),
    "wg_rhs": (_i, [_vp, _i, _dp]),
    "wg_compute_dt": (_i, [_vp, _i, _dp]),
    "wg_rk4_step": (_i, [_vp, _i, _dp, _dp]),
    "wg_run": (_i, [_vp, _i, _ip, _i, _i]),
    "wg_threshold_flags": (_i, [_vp, _i, _dp, _ip, _dp]),
    "wg_threshold_flags_wd": (_i, [_vp, _i, _dp, _ip, _dp]),
    "wg_refine_everywhere": (_i, [_vp, _i]),
    "wg_refine_significant": (_i, [_vp, _i]),
    "wg_get_refinement_status": (_i, [_vp, _i, _i, _ip]),
    "wg_set_refinement_status": (_i, [_vp, _i, _i, _ip]),
    "wg_sync_table": (_i, [_vp, _i, _i, _i, _i, _i, _ip]),
    "wg_block_slot": (_i, [_vp, _i, _i]),
    "wg_sync_table_host": (_i, [ctypes.POINTER(WgConfig), _i, _ip, _ip, _i, _i, _i, _i, _ip]),
    "wg_time_kernel": (_i, [_vp, _i, _i, _i, _dp]),
    "wg_tree_stats": (_i, [_vp, _i, _ip, _ip]),
    "wg_set_mask_sparse": (_i, [_vp, _i, _i, _ip, _dp]),
    "wg_set_mask_sphere": (_i, [_vp, _i, _dp, ctypes.c_double, ctypes.c_double]),
    "wg_get_mask_block": (_i, [_vp, _i, _i, _dp]),
    "wg_upload_interior": (_i, [_vp, _i, _dp]),
    "wg_download_interior": (_i, [_vp, _i, _dp]),
    "wg_graph_kernels": (_i, [_vp]),
    "wg_threshold_flags_noalloc": (_i, [ctypes.POINTER(WgConfig), _i, _vp, _dp, _vp, _vp, _vp]),
    "wg_set_geometry": (_i, [_vp, _i, ctypes.POINTER(WgGeometry)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m wabbit_gb300.build` "
                               "(the GB300 hot path has no CPU fallback)")
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code):
    if isinstance(code, int) and code < 0:
        msg = load().wg_last_error()
        raise WgError(code, msg.decode() if msg else "")
    return code
