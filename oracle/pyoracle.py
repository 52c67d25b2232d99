"""ctypes front-end of the CPU oracle (oracle/wg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from wabbit_gb300.config import WgConfig

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle library (make -C oracle)."""
    src = os.path.join(HERE, "wg_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [ctypes.POINTER(WgConfig)]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_set_grid.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _ip, _dp]
        L.or_nblocks.argtypes = [ctypes.c_void_p]
        L.or_get_grid.argtypes = [ctypes.c_void_p, _ip, _ip]
        L.or_get_data.argtypes = [ctypes.c_void_p, _dp]
        L.or_set_data.argtypes = [ctypes.c_void_p, _dp]
        L.or_set_mask.argtypes = [ctypes.c_void_p, _dp]
        L.or_set_mask_sparse.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp]
        L.or_set_interior.argtypes = [ctypes.c_void_p, _dp]
        L.or_get_neighbors.argtypes = [ctypes.c_void_p, _ip]
        L.or_sync_ghosts.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_sync_ghosts.restype = ctypes.c_int
        L.or_rhs.argtypes = [ctypes.c_void_p, _dp]
        L.or_dt.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        L.or_timestep.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_threshold_flags.argtypes = [ctypes.c_void_p, _dp, _ip, _dp]
        L.or_fwt.argtypes = [ctypes.c_void_p, _dp]
        L.or_iwt.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_adapt.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
        L.or_wc_threshold.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_refine_everywhere.argtypes = [ctypes.c_void_p]
        L.or_refine_significant.argtypes = [ctypes.c_void_p]
        L.or_set_coarse_extension.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_status.argtypes = [ctypes.c_void_p, _ip]
        L.or_set_status.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip]
        L.or_set_fd_stencil.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_filter.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _ip, _dp]
        L.or_adapt_full_tree.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
        L.or_run.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.or_set_geometry.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.or_make_mask.argtypes = [ctypes.c_void_p]
        L.or_get_mask.argtypes = [ctypes.c_void_p, _dp]
        L.or_mask_status.argtypes = [ctypes.c_void_p, _ip]
        L.or_norm.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        _lib = L
    return _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


class Oracle:
    """One oracle forest (blocks + state) for a given configuration."""

    def __init__(self, cfg: WgConfig, threads: int = 1):
        self.cfg = cfg.copy()
        self.L = lib()
        self.h = self.L.or_create(ctypes.byref(self.cfg))
        if not self.h:
            raise ValueError("oracle: unsupported configuration")
        self.L.or_set_threads(self.h, threads)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_destroy(self.h)
            self.h = None

    @property
    def block_shape(self):
        c = self.cfg
        return (c.neq, c.nz, c.Bs[1] + 2 * c.g, c.nx)

    def set_grid(self, level, coords, data=None):
        level = np.ascontiguousarray(level, np.int32)
        coords = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        n = len(level)
        d = None
        if data is not None:
            data = np.ascontiguousarray(data, np.float64).reshape((n,) + self.block_shape)
            d = _p(data)
        self.L.or_set_grid(self.h, n, _p(level, ctypes.c_int), _p(coords, ctypes.c_int), d)

    @property
    def nblocks(self):
        return self.L.or_nblocks(self.h)

    def grid(self):
        n = self.nblocks
        lv = np.zeros(n, np.int32)
        co = np.zeros((n, 3), np.int32)
        self.L.or_get_grid(self.h, _p(lv, ctypes.c_int), _p(co, ctypes.c_int))
        return lv, co

    def data(self):
        out = np.zeros((self.nblocks,) + self.block_shape)
        self.L.or_get_data(self.h, _p(out))
        return out

    def set_data(self, data):
        data = np.ascontiguousarray(data, np.float64)
        assert data.size == self.nblocks * int(np.prod(self.block_shape))
        self.L.or_set_data(self.h, _p(data))

    def set_mask(self, mask):
        if mask is None:
            self.L.or_set_mask(self.h, None)
        else:
            mask = np.ascontiguousarray(mask, np.float64)
            self.L.or_set_mask(self.h, _p(mask))

    def set_mask_sparse(self, ids, masks):
        """Masks (n, 6, nz, ny, nx) of the listed blocks; every other block
        has the all-zero mask."""
        ids = np.ascontiguousarray(ids, np.int32)
        masks = np.ascontiguousarray(masks, np.float64)
        assert masks.size == len(ids) * 6 * int(np.prod(self.block_shape[1:]))
        rc = self.L.or_set_mask_sparse(self.h, len(ids), _p(ids, ctypes.c_int), _p(masks))
        if rc != 0:
            raise RuntimeError(f"or_set_mask_sparse: {rc}")

    def set_interior(self, u):
        """Interior points of every block, (nblk, neq, Bz, By, Bx); the ghost
        nodes keep their values."""
        u = np.ascontiguousarray(u, np.float64)
        c = self.cfg
        bz = c.Bs[2] if c.dim == 3 else 1
        assert u.size == self.nblocks * c.neq * bz * c.Bs[1] * c.Bs[0]
        self.L.or_set_interior(self.h, _p(u))

    def set_geometry(self, geo):
        """Penalisation geometry (a WgGeometry) the masks are drawn from."""
        self.geo = geo
        self.L.or_set_geometry(self.h, ctypes.byref(geo) if geo is not None else None)

    def make_mask(self):
        """createMask_tree on the current grid (needs a geometry)."""
        self.L.or_make_mask(self.h)

    def mask(self):
        """The forest's masks (Nb, 6, nz, ny, nx), or None."""
        c = self.cfg
        out = np.zeros((self.nblocks, 6, c.nz, c.Bs[1] + 2 * c.g, c.nx))
        return out if self.L.or_get_mask(self.h, _p(out)) == 1 else None

    def mask_status(self):
        out = np.zeros(self.nblocks, np.int32)
        self.L.or_mask_status(self.h, _p(out, ctypes.c_int))
        return out

    def norm(self, which="Linfty"):
        """componentWiseNorm_tree over the leaves (per component)."""
        out = np.zeros(self.cfg.neq)
        self.L.or_norm(self.h, 0 if which == "Linfty" else 1, _p(out))
        return out

    def eps_use(self):
        """eps * norm per component as adapt_tree applies it with
        eps_normalized (norm <= 1e-9 is replaced by 1,
        coarseningIndicator_tree.f90:150-152), or eps without it."""
        if not self.cfg.eps_normalized:
            return np.full(self.cfg.neq, self.cfg.eps)
        n = self.norm("Linfty")
        n[n <= 1.0e-9] = 1.0
        return self.cfg.eps * n

    def neighbors(self):
        out = np.zeros((self.nblocks, 168), np.int32)
        self.L.or_get_neighbors(self.h, _p(out, ctypes.c_int))
        return out

    def sync(self, gminus=None, gplus=None, ignore_filter=True):
        gm = self.cfg.g_rhs if gminus is None else gminus
        gp = gm if gplus is None else gplus
        if self.L.or_sync_ghosts(self.h, gm, gp, 1 if ignore_filter else 0) != 0:
            raise ValueError("oracle: ghost widths out of range")

    def rhs(self):
        out = np.zeros((self.nblocks,) + self.block_shape)
        st = self.L.or_rhs(self.h, _p(out))
        if st:
            raise RuntimeError(f"oracle rhs status {st}")
        return out

    def dt(self, time):
        d = ctypes.c_double()
        self.L.or_dt(self.h, time, ctypes.byref(d))
        return d.value

    def step(self, time):
        t = ctypes.c_double(time)
        d = ctypes.c_double()
        st = self.L.or_timestep(self.h, ctypes.byref(t), ctypes.byref(d))
        if st:
            raise RuntimeError(f"oracle timestep status {st}")
        return t.value, d.value

    def run(self, nsteps, time):
        t = ctypes.c_double(time)
        dts = np.zeros(nsteps)
        n = self.L.or_run(self.h, nsteps, ctypes.byref(t), _p(dts))
        if n < 0:
            raise RuntimeError(f"oracle run status {n}")
        return t.value, dts[:n]

    def flags(self, eps_use):
        eps_use = np.ascontiguousarray(np.broadcast_to(eps_use, (self.cfg.neq,)), np.float64)
        fl = np.zeros(self.nblocks, np.int32)
        det = np.zeros((self.nblocks, self.cfg.neq))
        self.L.or_threshold_flags(self.h, _p(eps_use), _p(fl, ctypes.c_int), _p(det))
        return fl, det

    def fwt(self):
        out = np.zeros((self.nblocks,) + self.block_shape)
        self.L.or_fwt(self.h, _p(out))
        return out

    def iwt(self, wd):
        """IWT of every block from spaghetti data with synchronised ghosts
        (waveletReconstruction_optimized_block); ghosts copied through."""
        wd = np.ascontiguousarray(wd, np.float64)
        out = np.zeros_like(wd)
        self.L.or_iwt(self.h, _p(wd), _p(out))
        return out

    def wc_threshold(self, wd, thresh):
        """wc_threshold_tree on spaghetti data (returns a thresholded copy)."""
        out = np.array(wd, np.float64, copy=True, order="C")
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(thresh, np.float64), (self.cfg.neq,)))
        self.L.or_wc_threshold(self.h, _p(out), _p(t))
        return out

    def adapt(self, eps_use=None, everywhere=False):
        """adapt_tree (threshold-state-vector or everywhere); CDF X0 by
        decimation, CDF XY through the full tree with coarse extension and
        security zone; returns the new block count."""
        if everywhere:
            n = self.L.or_adapt(self.h, None, 1)
        else:
            e = np.ascontiguousarray(np.broadcast_to(np.asarray(eps_use, np.float64), (self.cfg.neq,)))
            n = self.L.or_adapt(self.h, _p(e), 0)
        if n < 0:
            raise RuntimeError(f"or_adapt failed ({n})")
        return n

    def adapt_full_tree(self, eps_use=None, everywhere=False):
        """adapt_tree through the full-tree path with coarse extension (the
        lifted-wavelet algorithm; for CDF X0 it reduces to the plain one)."""
        if everywhere:
            n = self.L.or_adapt_full_tree(self.h, None, 1)
        else:
            e = np.ascontiguousarray(np.broadcast_to(np.asarray(eps_use, np.float64), (self.cfg.neq,)))
            n = self.L.or_adapt_full_tree(self.h, _p(e), 0)
        if n < 0:
            raise RuntimeError(f"or_adapt_full_tree failed ({n})")
        return n

    def refine_everywhere(self):
        self.L.or_refine_everywhere(self.h)

    def refine_significant(self):
        """refine_tree with the "significant" indicator: the blocks the last
        adaptation found significant (and, for gradedness, their coarser
        neighbours) refine; returns the new block count."""
        n = self.L.or_refine_significant(self.h)
        if n < 0:
            raise RuntimeError(f"or_refine_significant failed ({n})")
        return n

    def status(self):
        """The leaves' refinement status after the last adaptation."""
        n = self.L.or_status(self.h, None)
        out = np.zeros(n, np.int32)
        if n:
            self.L.or_status(self.h, _p(out, ctypes.c_int))
        return out

    def set_status(self, st):
        """The leaves' refinement status (as read from a field file)."""
        st = np.ascontiguousarray(st, np.int32)
        if self.L.or_set_status(self.h, len(st), _p(st, ctypes.c_int)) != 0:
            raise RuntimeError("or_set_status: wrong length")

    def set_fd_stencil(self, n):
        """The FD stencil half-width of the wavelet set-up (0: none)."""
        if self.L.or_set_fd_stencil(self.h, int(n)) != 0:
            raise RuntimeError("or_set_fd_stencil failed")

    def set_coarse_extension(self, on=True):
        """useCoarseExtension and useSecurityZone for any wavelet."""
        self.L.or_set_coarse_extension(self.h, 1 if on else 0)

    def filter(self, which):
        lo, hi = ctypes.c_int(), ctypes.c_int()
        self.L.or_filter(self.h, which, ctypes.byref(lo), ctypes.byref(hi), None)
        c = np.zeros(hi.value - lo.value + 1)
        self.L.or_filter(self.h, which, ctypes.byref(lo), ctypes.byref(hi), _p(c))
        return lo.value, c


def pad_blocks(cfg: WgConfig, interior: np.ndarray) -> np.ndarray:
    """(Nb, nc, [Bs,] Bs, Bs) interiors -> (Nb, nc, nz, ny, nx) with zero ghosts."""
    g = cfg.g
    nb, nc = interior.shape[:2]
    out = np.zeros((nb, nc, cfg.nz, cfg.Bs[1] + 2 * g, cfg.nx))
    if cfg.dim == 2:
        out[:, :, 0, g:g + cfg.Bs[1], g:g + cfg.Bs[0]] = interior
    else:
        out[:, :, g:g + cfg.Bs[2], g:g + cfg.Bs[1], g:g + cfg.Bs[0]] = interior
    return out


def interior(cfg: WgConfig, full: np.ndarray) -> np.ndarray:
    g = cfg.g
    if cfg.dim == 2:
        return full[:, :, 0, g:g + cfg.Bs[1], g:g + cfg.Bs[0]]
    return full[:, :, g:g + cfg.Bs[2], g:g + cfg.Bs[1], g:g + cfg.Bs[0]]
