"""Host-side mirror of the reference's tree-level interface for the hot path.

The reference drives the time loop from Fortran (LIB/MAIN/main.f90:293-501)
through tree-level routines: sync_ghosts_RHS_tree, calculate_time_step,
timeStep_tree (-> RungeKuttaGeneric), coarseningIndicator_tree and
refine_tree. ``Forest`` exposes the same operations, backed by the CUDA
library; state lives on the device between calls.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .config import WgConfig


def probe_alu():
    """FP64 and FP32 FMA throughput of the current GPU in TFLOP/s, from the
    measurement library libwg_probe.so (not part of the product library)."""
    from . import build
    lib = ctypes.CDLL(build.build_probe())
    lib.wg_probe_alu.restype = ctypes.c_int
    lib.wg_probe_alu.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib.wg_probe_alu(ctypes.byref(a), ctypes.byref(b))
    if rc != 0:
        raise RuntimeError(f"wg_probe_alu: CUDA error {rc}")
    return a.value, b.value


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


class Context:
    """A device arena for one block geometry (the reference's allocate_forest)."""

    def __init__(self, cfg: WgConfig, max_blocks: int):
        self.L = capi.load()
        self.cfg = cfg.copy()
        h = ctypes.c_void_p()
        capi.check(self.L.wg_ctx_create(ctypes.byref(self.cfg), int(max_blocks), ctypes.byref(h)))
        self.h = h
        self.max_blocks = int(max_blocks)

    def close(self):
        if getattr(self, "h", None):
            self.L.wg_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_variant(self, fast: bool):
        capi.check(self.L.wg_set_variant(self.h, 1 if fast else 0))

    FORMS = {"auto": 0, "direct": 1, "tile": 2, "march": 3, "pipe": 4, "tile2": 5, "tile8": 6}

    def set_stage_form(self, form: str):
        """Form of the FP32-pipe stage kernel: auto (each RK stage timed in
        every applicable form before the first step), direct, tile (TMA-staged
        4-plane slabs) or march (whole blocks through a TMA plane ring)."""
        capi.check(self.L.wg_set_stage_form(self.h, self.FORMS[form]))

    def stage_form(self) -> str:
        f = ctypes.c_int()
        capi.check(self.L.wg_get_stage_form(self.h, ctypes.byref(f)))
        return {v: k for k, v in self.FORMS.items()}[f.value]

    def set_stage_forms(self, forms):
        """Fix the forms of RK stages 1-4 (names: direct, tile, march)."""
        f = (ctypes.c_int * 4)(*[self.FORMS[x] for x in forms])
        capi.check(self.L.wg_set_stage_forms(self.h, f))

    def stage_forms(self) -> list:
        """The forms of RK stages 1-4."""
        f = (ctypes.c_int * 4)()
        capi.check(self.L.wg_get_stage_forms(self.h, f))
        names = {v: k for k, v in self.FORMS.items()}
        return [names[x] for x in f]

    def synchronize(self):
        capi.check(self.L.wg_synchronize(self.h))

    def forest(self, cfg: WgConfig | None = None) -> "Forest":
        return Forest(self, cfg)

    def run(self, forests, nsteps: int, use_graph: bool = True):
        ids = np.array([f.tree for f in forests], np.int32)
        capi.check(self.L.wg_run(self.h, len(ids), _p(ids, ctypes.c_int), int(nsteps), 1 if use_graph else 0))

    PROFILE_KEYS = ("sync1", "sync2", "sync3", "sync4", "dt", "stage1", "stage2", "stage3", "stage4")

    def step_profile(self, forests, nsteps: int) -> dict:
        """Mean device time (ms) per RK4 step of each kernel group over
        nsteps profiled steps (the state advances)."""
        ids = np.array([f.tree for f in forests], np.int32)
        ms = np.zeros(9)
        capi.check(self.L.wg_step_profile(self.h, len(ids), _p(ids, ctypes.c_int), int(nsteps), _p(ms)))
        return dict(zip(self.PROFILE_KEYS, ms.tolist()))

    @property
    def stream(self) -> int:
        return self.L.wg_stream(self.h)


class Forest:
    """One tree (independent solve) inside a Context."""

    def __init__(self, ctx: Context, cfg: WgConfig | None = None):
        self.ctx = ctx
        self.L = ctx.L
        self.cfg = (cfg or ctx.cfg).copy()
        t = ctypes.c_int()
        capi.check(self.L.wg_tree_create(ctx.h, ctypes.byref(self.cfg), ctypes.byref(t)))
        self.tree = t.value

    def destroy(self):
        if self.tree >= 0 and self.ctx.h:
            capi.check(self.L.wg_tree_destroy(self.ctx.h, self.tree))
        self.tree = -1

    # ---------------------------------------------------------------- layout
    @property
    def block_shape(self):
        c = self.cfg
        return (c.neq, c.nz, c.Bs[1] + 2 * c.g, c.nx)

    @property
    def nblocks(self) -> int:
        n = ctypes.c_int()
        capi.check(self.L.wg_get_nblocks(self.ctx.h, self.tree, ctypes.byref(n)))
        return n.value

    def set_grid(self, level, coords):
        level = np.ascontiguousarray(level, np.int32)
        coords = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        capi.check(self.L.wg_set_grid(self.ctx.h, self.tree, len(level), _p(level, ctypes.c_int),
                                      _p(coords, ctypes.c_int)))

    def grid(self):
        n = self.nblocks
        lv = np.zeros(n, np.int32)
        co = np.zeros((n, 3), np.int32)
        capi.check(self.L.wg_get_grid(self.ctx.h, self.tree, n, _p(lv, ctypes.c_int), _p(co, ctypes.c_int)))
        return lv, co

    def upload(self, data):
        data = np.ascontiguousarray(data, np.float64)
        if data.size != self.nblocks * int(np.prod(self.block_shape)):
            raise ValueError("state has the wrong size for this grid")
        capi.check(self.L.wg_upload_state(self.ctx.h, self.tree, _p(data)))

    def download(self):
        out = np.zeros((self.nblocks,) + self.block_shape)
        capi.check(self.L.wg_download_state(self.ctx.h, self.tree, _p(out)))
        return out

    # ------------------------------------------------------------ files
    FIELD_NAMES = {2: ("ux", "uy", "p"), 3: ("ux", "uy", "uz", "p")}

    def save_hdf5(self, directory: str, iteration: int = 0, names=None) -> list:
        """save_data (LIB/IO/save_data.f90:1-90): one file per component,
        <name>_<timestr>.h5 in saveHDF5_tree's layout (interior plus the
        first ghost layer on the upper side, after a ghost sync of g
        layers). Returns the paths written."""
        import os

        from . import h5io
        c = self.cfg
        dim = c.dim
        names = names or self.FIELD_NAMES[dim]
        self.sync_ghosts_tree()
        full = self.download()                       # (Nb, neq, nz, ny, nx)
        lv, co = self.grid()
        t, _ = self.time()
        g = c.g
        sl = (slice(g, g + c.Bs[1] + 1), slice(g, g + c.Bs[0] + 1))
        if dim == 3:
            sl = (slice(g, g + c.Bs[2] + 1),) + sl
        out = []
        for k, name in enumerate(names):
            comp = full[:, k] if dim == 3 else full[:, k, 0]
            path = os.path.join(directory, f"{name}_{h5io.timestr(t)}.h5")
            h5io.save_wabbit(path, comp[(slice(None),) + sl], lv, co[:, :dim], t, iteration,
                             list(c.domain)[:dim], list(c.Bs)[:dim], c.Jmax)
            out.append(path)
        return out

    def load_hdf5(self, paths):
        """The grid, state and time from field files of one time stamp (one
        file per component, in component order), as the reference's
        readHDF5vct_tree does for a restart (LIB/MESH/InputOutput.f90:322)."""
        from . import h5io
        ds = [h5io.read_wabbit(p) for p in paths]
        if len(ds) != self.cfg.neq:
            raise ValueError(f"expected {self.cfg.neq} files, one per component")
        c = self.cfg
        lv, co = ds[0]["level"], ds[0]["coords"]
        for d in ds[1:]:
            if not (np.array_equal(d["level"], lv) and np.array_equal(d["coords"], co)):
                raise ValueError("the files hold different grids")
        if list(ds[0]["Bs"]) != list(c.Bs)[:c.dim]:
            raise ValueError("block size of the files differs from the configuration")
        co3 = np.zeros((len(lv), 3), np.int32)
        co3[:, :c.dim] = co
        self.set_grid(lv, co3)
        inner = tuple(slice(0, b) for b in list(c.Bs)[:c.dim][::-1])
        u = np.stack([d["blocks"][(slice(None),) + inner] for d in ds], axis=1)
        if c.dim == 2:
            u = u[:, :, None]
        self.upload_interior(np.ascontiguousarray(u))
        self.set_time(ds[0]["time"])
        return ds[0]["iteration"]

    @property
    def interior_shape(self):
        c = self.cfg
        return (c.neq, c.Bs[2] if c.dim == 3 else 1, c.Bs[1], c.Bs[0])

    def upload_interior(self, data):
        """Interior state (nblk, neq, Bz, By, Bx) from a numpy array or a
        contiguous float64 CUDA tensor (device memory is copied on the
        device after the tensor's stream has finished writing it)."""
        n = self.nblocks * int(np.prod(self.interior_shape))
        if hasattr(data, "data_ptr") and getattr(data, "is_cuda", False):
            import torch
            if data.dtype != torch.float64 or not data.is_contiguous() or data.numel() != n:
                raise ValueError("device interior state must be a contiguous float64 tensor of the grid's size")
            torch.cuda.current_stream(data.device).synchronize()
            ptr = ctypes.cast(ctypes.c_void_p(data.data_ptr()), ctypes.POINTER(ctypes.c_double))
            capi.check(self.L.wg_upload_interior(self.ctx.h, self.tree, ptr))
            return
        data = np.ascontiguousarray(data, np.float64)
        if data.size != n:
            raise ValueError("interior state has the wrong size for this grid")
        capi.check(self.L.wg_upload_interior(self.ctx.h, self.tree, _p(data)))

    def download_interior(self, out=None):
        if out is None:
            out = np.zeros((self.nblocks,) + self.interior_shape)
        capi.check(self.L.wg_download_interior(self.ctx.h, self.tree, _p(out)))
        return out

    def rk4_stream(self, ins, outs):
        """len(ins) RK4 steps with host buffers (wg_rk4_stream): step k starts
        from the interior state ins[k] and writes its result to outs[k];
        page-locked buffers let the transfers overlap the steps."""
        if len(ins) != len(outs):
            raise ValueError("ins and outs differ in length")
        n = self.nblocks * int(np.prod(self.interior_shape))
        for a in list(ins) + list(outs):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != n:
                raise ValueError("buffers must be contiguous float64 arrays of the interior size")
        pin = (ctypes.POINTER(ctypes.c_double) * len(ins))(*[_p(a) for a in ins])
        pout = (ctypes.POINTER(ctypes.c_double) * len(outs))(*[_p(a) for a in outs])
        capi.check(self.L.wg_rk4_stream(self.ctx.h, self.tree, len(ins), pin, pout))

    def set_mask(self, mask):
        if mask is None:
            capi.check(self.L.wg_set_mask(self.ctx.h, self.tree, None))
            return
        mask = np.ascontiguousarray(mask, np.float64)
        c = self.cfg
        if mask.size != self.nblocks * 6 * c.npts:
            raise ValueError("mask has the wrong size")
        capi.check(self.L.wg_set_mask(self.ctx.h, self.tree, _p(mask)))

    def set_mask_sparse(self, blocks, mask):
        blocks = np.ascontiguousarray(blocks, np.int32)
        mask = np.ascontiguousarray(mask, np.float64)
        if mask.size != len(blocks) * 6 * self.cfg.npts:
            raise ValueError("mask has the wrong size")
        capi.check(self.L.wg_set_mask_sparse(self.ctx.h, self.tree, len(blocks), _p(blocks, ctypes.c_int), _p(mask)))

    def set_geometry(self, geo):
        """Penalisation geometry (config.WgGeometry) the tree draws its masks
        from after every grid change, as createMask_tree does; None removes
        it."""
        capi.check(self.L.wg_set_geometry(self.ctx.h, self.tree, ctypes.byref(geo) if geo is not None else None))

    def set_mask_sphere(self, centre, radius, c_smooth=1.5):
        """Fixed-sphere penalisation mask computed on the device (3-D)."""
        c = np.ascontiguousarray(centre, np.float64)
        capi.check(self.L.wg_set_mask_sphere(self.ctx.h, self.tree, _p(c), float(radius), float(c_smooth)))

    def mask_block(self, block):
        """Interior mask (6, Bz, By, Bx) of a block, or None without one."""
        Bz = self.cfg.Bs[2] if self.cfg.dim == 3 else 1
        out = np.zeros((6, Bz, self.cfg.Bs[1], self.cfg.Bs[0]))
        r = capi.check(self.L.wg_get_mask_block(self.ctx.h, self.tree, int(block), _p(out)))
        return out if r == 1 else None

    def stats(self):
        n, m = ctypes.c_int(), ctypes.c_int()
        capi.check(self.L.wg_tree_stats(self.ctx.h, self.tree, ctypes.byref(n), ctypes.byref(m)))
        return n.value, m.value

    def time_kernel(self, which: int, reps: int = 20) -> float:
        ms = ctypes.c_double()
        capi.check(self.L.wg_time_kernel(self.ctx.h, self.tree, which, reps, ctypes.byref(ms)))
        return ms.value

    # ------------------------------------------------------------------ time
    def set_time(self, t: float):
        capi.check(self.L.wg_set_time(self.ctx.h, self.tree, float(t)))

    def time(self):
        t, d = ctypes.c_double(), ctypes.c_double()
        capi.check(self.L.wg_get_time(self.ctx.h, self.tree, ctypes.byref(t), ctypes.byref(d)))
        return t.value, d.value

    # -------------------------------------------------------- reference ops
    def sync_ghosts_RHS_tree(self, g_minus=None, g_plus=None):
        gm = self.cfg.g_rhs if g_minus is None else g_minus
        gp = gm if g_plus is None else g_plus
        capi.check(self.L.wg_sync_ghosts(self.ctx.h, self.tree, gm, gp))

    def sync_ghosts_tree(self):
        """Full ghost sync with g layers (CDFX0 wavelets: no HD filter)."""
        capi.check(self.L.wg_sync_ghosts(self.ctx.h, self.tree, self.cfg.g, self.cfg.g))

    def RHS_ACM(self):
        out = np.zeros((self.nblocks,) + self.block_shape)
        capi.check(self.L.wg_rhs(self.ctx.h, self.tree, _p(out)))
        return out

    def calculate_time_step(self) -> float:
        d = ctypes.c_double()
        capi.check(self.L.wg_compute_dt(self.ctx.h, self.tree, ctypes.byref(d)))
        return d.value

    def timeStep_tree(self):
        """One RK4 step; returns (time, dt) after the step."""
        t, d = ctypes.c_double(), ctypes.c_double()
        capi.check(self.L.wg_rk4_step(self.ctx.h, self.tree, ctypes.byref(t), ctypes.byref(d)))
        return t.value, d.value

    def run(self, nsteps: int, use_graph: bool = True):
        self.ctx.run([self], nsteps, use_graph)

    def coarseningIndicator(self, eps_use, input_is_wd: bool = False):
        """Flags (-1 may coarsen, 0 stay) and per-component details; with
        input_is_wd the state already holds the decomposition."""
        eps_use = np.ascontiguousarray(np.broadcast_to(np.asarray(eps_use, np.float64), (self.cfg.neq,)))
        n = self.nblocks
        flags = np.zeros(n, np.int32)
        det = np.zeros((n, self.cfg.neq))
        fn = self.L.wg_threshold_flags_wd if input_is_wd else self.L.wg_threshold_flags
        capi.check(fn(self.ctx.h, self.tree, _p(eps_use), _p(flags, ctypes.c_int), _p(det)))
        return flags, det

    def wavelet_decompose(self):
        """One-level FWT of every block in place (spaghetti order); ghosts
        must be synchronised first (sync_ghosts_tree)."""
        capi.check(self.L.wg_wavelet_decompose(self.ctx.h, self.tree))

    def wavelet_reconstruct(self):
        """One-level IWT of every block in place; the ghosts must hold the
        neighbours' decomposed data."""
        capi.check(self.L.wg_wavelet_reconstruct(self.ctx.h, self.tree))

    def wc_threshold(self, thresh):
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(thresh, np.float64), (self.cfg.neq,)))
        capi.check(self.L.wg_wavelet_threshold(self.ctx.h, self.tree, _p(t)))

    def adapt(self, eps_use=None, everywhere: bool = False) -> int:
        """adapt_tree (coarsening) with the threshold-state-vector indicator
        (eps_use = eps * norm per component; None: the configuration's eps,
        normalised by the leaves' Linfty norm with eps_normalized) or on
        every leaf. CDF X0: full tree by decimation; CDF XY: full-tree FWT
        with coarse extension, security zone and reconstruction at the
        coarse/fine interfaces. Replaces grid and state, redraws the masks
        from the geometry (else drops them), returns the new block count."""
        n = ctypes.c_int()
        if everywhere:
            capi.check(self.L.wg_adapt(self.ctx.h, self.tree, None, 1, ctypes.byref(n)))
        elif eps_use is None:
            capi.check(self.L.wg_adapt(self.ctx.h, self.tree, None, 0, ctypes.byref(n)))
        else:
            e = np.ascontiguousarray(np.broadcast_to(np.asarray(eps_use, np.float64), (self.cfg.neq,)))
            capi.check(self.L.wg_adapt(self.ctx.h, self.tree, _p(e), 0, ctypes.byref(n)))
        return n.value

    def adapt_profile(self, enable=None):
        """Phase times (ms) of the last lifted adaptation: planning, syncs,
        FWT, coarse extension + D2M, indicator + security zone, IWT, block
        copies, total; enable switches the phase timing for later calls."""
        out = np.zeros(8)
        capi.check(self.L.wg_adapt_profile(self.ctx.h, -1 if enable is None else int(bool(enable)), _p(out), 8))
        return dict(zip(("plan", "sync", "fwt", "ce_d2m", "flags", "iwt", "copy", "total"), out.tolist()))

    def refine_everywhere(self):
        capi.check(self.L.wg_refine_everywhere(self.ctx.h, self.tree))

    def refine_significant(self):
        """refine_tree(..., "significant"): the blocks the last adaptation
        found significant refine (and, for gradedness, their coarser
        neighbours)."""
        capi.check(self.L.wg_refine_significant(self.ctx.h, self.tree))

    def set_refinement_status(self, status):
        """The status of the current blocks as a restarted run reads it."""
        st = np.ascontiguousarray(status, np.int32)
        capi.check(self.L.wg_set_refinement_status(self.ctx.h, self.tree, len(st), _p(st, ctypes.c_int)))

    def refinement_status(self):
        """The status the last adaptation left per block (0 or 9)."""
        n = capi.check(self.L.wg_get_refinement_status(self.ctx.h, self.tree, 0, None))
        out = np.zeros(n, np.int32)
        capi.check(self.L.wg_get_refinement_status(self.ctx.h, self.tree, n, _p(out, ctypes.c_int)))
        return out

    def sync_table(self, gminus, gplus, thin=False):
        n = capi.check(self.L.wg_sync_table(self.ctx.h, self.tree, gminus, gplus, 1 if thin else 0, 0, None))
        out = np.zeros((n, 19), np.int32)
        capi.check(self.L.wg_sync_table(self.ctx.h, self.tree, gminus, gplus, 1 if thin else 0, n,
                                        _p(out, ctypes.c_int)))
        return out
