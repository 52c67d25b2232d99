"""The reference's 2-D cylinder regression case (TESTING/acm/acm_CDF40 and
acm_CDF44) as test data: configuration and geometry from the stored
acm_cyl.ini text, the stored states and masks, and the reference's main loop
(LIB/MAIN/main.f90:293-427: sync_ghosts_tree, refine_tree everywhere,
timeStep_tree, adapt_tree, every iteration) driven through the oracle or the
library."""
import numpy as np

from wabbit_gb300 import config

TAGS = {"t0": 0.0, "t1": 0.05, "t2": 0.1}


class Case:
    def __init__(self, golden, wavelet):
        z = golden("acm_cyl.npz")
        self.w = wavelet
        self.z = {k[len(wavelet) + 1:]: z[k] for k in z.files if k.startswith(wavelet + "_")}
        ini = str(self.z["ini"])
        self.cfg = config.from_ini_text(ini)
        self.geo = config.geometry_from_ini_text(ini, self.cfg)
        kv = config._parse_ini(ini)
        # refine_tree's indicator of the main loop (main.f90:309-330)
        self.significant = kv.get(("Blocks", "refinement_indicator"), "everywhere").strip() == "significant"

    def status(self, key):
        return self.z[f"{key}_status"]

    def grid(self, key):
        return self.z[f"{key}_level"], self.z[f"{key}_coords"]

    def state(self, key):
        return self.z[f"{key}_u"]

    def chi(self, key):
        return self.z[f"{key}_chi"]

    def iteration(self, key):
        return int(self.z[f"{key}_iteration"])


def reorder(lv_ref, co_ref, lv, co):
    """Permutation taking grid (lv, co) to the order of (lv_ref, co_ref), or
    None if the two grids differ."""
    k_ref = [(int(l), *map(int, c)) for l, c in zip(lv_ref, co_ref)]
    k = {(int(l), *map(int, c)): i for i, (l, c) in enumerate(zip(lv, co))}
    if set(k_ref) != set(k) or len(k) != len(k_ref):
        return None
    return np.array([k[x] for x in k_ref])


def run_oracle(case, tend, threads=1):
    """The reference's loop in the oracle from the stored t=0 state until
    t = tend; returns (oracle, iterations, time)."""
    from pyoracle import Oracle, pad_blocks

    cfg = case.cfg
    o = Oracle(cfg, threads=threads)
    lv, co = case.grid("t0")
    o.set_grid(lv, co, pad_blocks(cfg, case.state("t0")))
    o.set_geometry(case.geo)
    if case.significant:   # the status the initial adaptation left, saved with the t=0 state
        o.set_status(case.status("t0"))
    t, it = 0.0, 0
    while t < tend - 1e-12:
        o.sync(cfg.g, cfg.g, ignore_filter=True)
        if case.significant:
            o.refine_significant()
        else:
            o.refine_everywhere()
        o.make_mask()
        t, _ = o.step(t)
        o.adapt(o.eps_use())
        it += 1
    return o, it, t


def run_library(case, tend, fast=False, precision=0, max_blocks=1200):
    """The same loop through the C ABI (wabbit_gb300.solver); the tree draws
    its masks from the geometry and normalises eps itself. Returns
    (grid, interior state, iterations, time)."""
    from pyoracle import interior, pad_blocks
    from wabbit_gb300.solver import Context

    cfg = case.cfg.copy()
    cfg.rhs_precision = precision
    lv, co = case.grid("t0")
    with Context(cfg, max_blocks) as ctx:
        ctx.set_variant(fast)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(pad_blocks(cfg, case.state("t0")))
        f.set_geometry(case.geo)
        f.set_time(0.0)
        if case.significant:
            f.set_refinement_status(case.status("t0"))
        t, it = 0.0, 0
        while t < tend - 1e-12:
            f.sync_ghosts_tree()
            if case.significant:
                f.refine_significant()
            else:
                f.refine_everywhere()
            t, _ = f.timeStep_tree()
            f.adapt()
            it += 1
        glv, gco = f.grid()
        u = interior(cfg, f.download())
    return (glv, gco), u, it, t
