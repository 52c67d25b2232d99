"""Serving loop: independent ACM solves admitted as they arrive, batched on
the device.

Requests are independent solves (the reference's tree_ID, LIB/MESH/forest.f90:
one tree per solve) of one of two block geometries: 2-D (Bs=16, CDF4,0, g=4)
or 3-D (Bs=16^3, CDF4,4, g=6). Each geometry has one context whose arena is
sized from an HBM budget. The loop

* admits queued requests first come first served per geometry as soon as
  the arena has free slots for their blocks (admission by HBM footprint),
* serves each geometry from its own host thread (one context per thread,
  the documented threading model): the 2-D and 3-D rounds, adaptations and
  admissions run independently, and the two contexts' kernels overlap on
  their own streams; a new arrival waits at most for the end of the current
  round (one chunk) of its geometry,
* steps every active solve of a context with one wg_run per scheduling
  round: one launch per kernel for all of them (batched FP32-pipe stages),
* adapts the grids every `adapt_every` steps as the reference's main loop
  does (LIB/MAIN/main.f90:300-400: ghost sync, refine_tree "everywhere",
  N_dt_per_grid time steps, adapt_tree with the threshold-state-vector
  indicator, absolute eps): every chunk of a solve is one such cycle; the
  3-D solves (CDF4,4) take the lifted full-tree adaptation. A request's Jmax
  is the finest level of its initial grid. A solve takes part in a round
  only if the arena can hold its refined grid plus the full tree's mothers;
  otherwise it waits for the next round,
* retires solves that reached their step count (downloads the interior
  state, frees the slots) and records the time to solution.

A solve's result does not depend on which other solves share its launches
(every kernel works per block and per tree), so a solve served in the mix is
bit-identical to the same solve run alone with the same step chunks.

Synthetic stream (seeded): Poisson arrivals; half 2-D, half 3-D; grid sizes
from a ladder spanning 64-2048 (2-D) and 512-8192 (3-D) blocks; Gaussian
velocity-vortex initial conditions (2-D: point vortices; 3-D: vortex tubes
with a uniformly random axis), nu ~ U[5e-4, 5e-3], p = 0, periodic unit
domain, no mask.
"""
from __future__ import annotations

import dataclasses
import threading
import time

import numpy as np

from . import config, grids
from .solver import Context

# block-count ladders of the request grids (level jmin equidistant, refined
# around a ball with the given radius at the next levels)
LADDER = {
    2: [(3, 3, 0.0), (3, 4, 0.22), (4, 4, 0.0), (4, 5, 0.18), (5, 5, 0.0), (5, 6, 0.3)],        # 64 .. 2020
    3: [(3, 3, 0.0), (3, 4, 0.22), (3, 4, 0.32), (4, 4, 0.0), (4, 5, 0.17), (4, 5, 0.26)],     # 512 .. ~7700
}


def geometry(dim: int):
    c = config.defaults(dim)
    for d in range(dim):
        c.Bs[d] = 16
    c.domain[0] = c.domain[1] = c.domain[2] = 1.0
    if dim == 2:
        c.wavelet, c.g, c.g_rhs = b"CDF40", 4, 2
    else:
        c.wavelet, c.g, c.g_rhs = b"CDF44", 6, 2
    c.Jmin, c.Jmax = 2, 7
    c.c0, c.gamma_p = (20.0 if dim == 2 else 15.0), 1.0
    c.penalization = 0
    c.CFL = 0.5
    c.time_max = 1e9
    c.rhs_precision = 1
    return c


_grid_cache: dict = {}


def request_grid(dim: int, size: int):
    key = (dim, size)
    if key not in _grid_cache:
        jmin, jmax, r = LADDER[dim][size]
        if jmax == jmin:
            lv, co = grids.equidistant(dim, jmin)
        else:
            lv, co = grids.refined_around(dim, jmin, jmax, [1.0, 1.0, 1.0], [0.5, 0.5, 0.5],
                                          lambda l, r=r: r)
        _grid_cache[key] = (lv, co)
    return _grid_cache[key]


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float      # seconds after the start of the stream
    dim: int
    size: int           # index into LADDER[dim]
    seed: int
    nu: float
    nsteps: int = 50


def make_stream(n: int = 256, rate: float = 8.0, seed: int = 4, nsteps: int = 50, dims=(2, 3)):
    """Seeded Poisson stream of n requests (rate per second)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        dim = int(dims[rng.integers(len(dims))])
        out.append(Request(i, float(t[i]), dim, int(rng.integers(len(LADDER[dim]))), int(rng.integers(1 << 31)),
                           float(rng.uniform(5e-4, 5e-3)), nsteps))
    return out


def vortex_ic(cfg, lv, co, seed: int, nvort: int = 6):
    """Interior IC (nblk, neq, Bz, By, Bx): Gaussian velocity vortices
    u = G/(pi R^2) exp(-r^2/R^2) (axis x r) with minimum-image distances on
    the unit torus; 2-D: axis = z; 3-D: tubes with a random unit axis."""
    rng = np.random.default_rng(seed)
    dim = cfg.dim
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, dim)
    Bx, By = cfg.Bs[0], cfg.Bs[1]
    Bz = cfg.Bs[2] if dim == 3 else 1
    nb = len(lv)
    X = x0[:, 0, None, None, None] + np.arange(Bx)[None, None, None, :] * dx[:, 0, None, None, None]
    Y = x0[:, 1, None, None, None] + np.arange(By)[None, None, :, None] * dx[:, 1, None, None, None]
    Z = (x0[:, 2, None, None, None] + np.arange(Bz)[None, :, None, None] * dx[:, 2, None, None, None]
         if dim == 3 else np.zeros((nb, 1, 1, 1)))
    u = np.zeros((nb, dim + 1, Bz, By, Bx))
    for _ in range(nvort):
        c = rng.uniform(0.0, 1.0, size=3)
        R = rng.uniform(0.05, 0.12)
        G = rng.normal(0.0, 1.0)
        a = np.array([0.0, 0.0, 1.0])
        if dim == 3:
            a = rng.normal(size=3)
            a /= np.linalg.norm(a)
        r = [X - c[0], Y - c[1], Z - c[2] if dim == 3 else np.zeros_like(X)]
        r = [q - np.rint(q) for q in r]
        ra = r[0] * a[0] + r[1] * a[1] + r[2] * a[2]
        rp = [r[k] - ra * a[k] for k in range(3)]
        amp = G / (np.pi * R * R) * np.exp(-(rp[0] ** 2 + rp[1] ** 2 + rp[2] ** 2) / (R * R))
        # a x r_perp
        cr = [a[1] * rp[2] - a[2] * rp[1], a[2] * rp[0] - a[0] * rp[2], a[0] * rp[1] - a[1] * rp[0]]
        for k in range(dim):
            u[:, k] += amp * cr[k]
    return u


def vortex_ic_device(cfg, lv, co, seed: int, nvort: int = 6):
    """vortex_ic evaluated on the GPU (torch, float64): the same vortex
    parameters (drawn on the host from the seed), the arithmetic on the
    device so that large requests are set up in milliseconds."""
    import torch
    rng = np.random.default_rng(seed)
    dim = cfg.dim
    dev = torch.device("cuda")
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, dim)
    x0 = torch.as_tensor(x0, device=dev)
    dx = torch.as_tensor(dx, device=dev)
    Bx, By = cfg.Bs[0], cfg.Bs[1]
    Bz = cfg.Bs[2] if dim == 3 else 1
    nb = len(lv)
    ar = lambda n: torch.arange(n, device=dev, dtype=torch.float64)
    X = x0[:, 0, None, None, None] + ar(Bx)[None, None, None, :] * dx[:, 0, None, None, None]
    Y = x0[:, 1, None, None, None] + ar(By)[None, None, :, None] * dx[:, 1, None, None, None]
    Z = (x0[:, 2, None, None, None] + ar(Bz)[None, :, None, None] * dx[:, 2, None, None, None]
         if dim == 3 else torch.zeros((nb, 1, 1, 1), device=dev, dtype=torch.float64))
    u = torch.zeros((nb, dim + 1, Bz, By, Bx), device=dev, dtype=torch.float64)
    for _ in range(nvort):
        c = rng.uniform(0.0, 1.0, size=3)
        R = rng.uniform(0.05, 0.12)
        G = rng.normal(0.0, 1.0)
        a = np.array([0.0, 0.0, 1.0])
        if dim == 3:
            a = rng.normal(size=3)
            a /= np.linalg.norm(a)
        r = [X - c[0], Y - c[1], Z - c[2] if dim == 3 else torch.zeros_like(X)]
        r = [q - torch.round(q) for q in r]
        ra = r[0] * a[0] + r[1] * a[1] + r[2] * a[2]
        rp = [r[k] - ra * a[k] for k in range(3)]
        amp = G / (np.pi * R * R) * torch.exp(-(rp[0] ** 2 + rp[1] ** 2 + rp[2] ** 2) / (R * R))
        cr = [a[1] * rp[2] - a[2] * rp[1], a[2] * rp[0] - a[0] * rp[2], a[0] * rp[1] - a[1] * rp[0]]
        for k in range(dim):
            u[:, k] += amp * cr[k]
    return u


class Solve:
    """One admitted request: its tree in the context of its geometry."""

    def __init__(self, req: Request, ctx: Context, base):
        self.req = req
        cfg = base.copy()
        cfg.nu = req.nu
        cfg.Jmax = LADDER[req.dim][req.size][1]
        self.cfg = cfg
        lv, co = request_grid(req.dim, req.size)
        self.nblk = len(lv)
        self.f = ctx.forest(cfg)
        self.f.set_grid(lv, co)
        self.f.upload_interior(vortex_ic_device(cfg, lv, co, req.seed))
        self.f.set_time(0.0)
        self.done = 0
        self.pts_blk = int(np.prod([cfg.Bs[d] for d in range(cfg.dim)]))

    @property
    def points(self):
        return self.nblk * self.pts_blk

    def cycle_need(self):
        """Blocks of the refined grid and of the full tree's mothers of the
        next adaptation cycle (upper bound)."""
        lv, _ = self.f.grid()
        nd = 1 << self.cfg.dim
        refined = int(np.sum(np.where(lv < self.cfg.Jmax, nd, 1)))
        return refined, refined // (nd - 1) + 2 * (self.cfg.Jmax + 1)

    def cycle(self):
        """Before a chunk: sync and refine everywhere (main.f90:300-320)."""
        self.f.sync_ghosts_tree()
        self.f.refine_everywhere()
        self.nblk = self.f.nblocks


class _Worker:
    """One context of a geometry with the solves it is stepping."""

    def __init__(self, dim: int, ctx: Context):
        self.dim = dim
        self.ctx = ctx
        self.capacity = ctx.max_blocks
        self.pinned = None

    def result_buffer(self, n):
        """Pinned host buffer of n doubles for a finished solve's state
        (grown on demand and reused: the download runs at copy-engine speed
        and touches no fresh pages)."""
        t = self.pinned
        if t is None or t.numel() < n:
            import torch
            t = torch.empty(max(n, int(1.25 * (t.numel() if t is not None else 0))), dtype=torch.float64,
                            pin_memory=True)
            self.pinned = t
        return t.numpy()[:n]


class Server:
    """workers: contexts (each served by its own host thread) per geometry.
    With several contexts of one geometry the first is sized for the largest
    request's peak and the others share the rest of the geometry's budget;
    each takes the earliest waiting request that fits its free slots (the
    large context takes small requests only while no large one waits), so
    the adaptations and admissions of different contexts overlap."""

    def __init__(self, budget_gb: float = 64.0, chunk: int = 5, share_3d: float = 0.85, keep_results=False,
                 adapt_every: int = 0, eps: float = 1e-3, workers=None):
        from . import capi
        self.chunk = adapt_every if adapt_every else chunk
        self.adapt = bool(adapt_every)
        self.eps = eps
        self.keep = keep_results
        self.base = {2: geometry(2), 3: geometry(3)}
        workers = dict(workers or {3: 2, 2: 1})
        L = capi.load()
        self.workers = {}
        for dim, share in ((3, share_3d), (2, 1.0 - share_3d)):
            per = L.wg_bytes_per_block(self.base[dim])
            if self.adapt and self.base[dim].wavelet.decode()[4] != "0":
                # the lifted adaptation's hvy_tmp arena: one more full block
                c = self.base[dim]
                per += 8 * c.neq * int(np.prod([c.Bs[d] + 2 * c.g for d in range(dim)]))
            total = budget_gb * 1e9 * share / per
            n = max(1, int(workers.get(dim, 1)))
            if n == 1:
                caps = [total]
            else:
                # the largest request peak that the whole budget can hold
                needs = [self._need(dim, Request(0, 0.0, dim, k, 0, 1e-3)) for k in range(len(LADDER[dim]))]
                big = max([x for x in needs if 1.02 * x <= total] or [0])
                first = min(total, max(total / n, 1.02 * big))
                caps = [first] + [max(0.0, (total - first) / (n - 1))] * (n - 1)
            self.workers[dim] = [_Worker(dim, Context(self.base[dim], max(64, int(c)))) for c in caps]
        self.capacity = {d: max(w.capacity for w in ws) for d, ws in self.workers.items()}
        self.ctx = {d: ws[0].ctx for d, ws in self.workers.items()}

    def _peak(self, dim, req):
        """Blocks a request needs at the peak of its first cycle."""
        lv, _ = request_grid(dim, req.size)
        nd = 1 << dim
        refined = int(np.sum(np.where(lv < LADDER[dim][req.size][1], nd, 1)))
        return refined + refined // (nd - 1) + 2 * (LADDER[dim][req.size][1] + 1)

    def _need(self, dim, req):
        return self._peak(dim, req) if self.adapt else len(request_grid(dim, req.size)[0])

    def warm_up(self):
        """One small solve of 5 steps (one adaptation cycle) on every context:
        graph capture and the stage-kernel autotuner happen here, not in the
        first served requests."""
        for dim, ws in self.workers.items():
            for w in ws:
                s = Solve(Request(-1, 0.0, dim, 0, 1, 1e-3, nsteps=self.chunk), w.ctx, self.base[dim])
                if self.adapt:
                    s.cycle()
                w.ctx.run([s.f], self.chunk, use_graph=True)
                if self.adapt:
                    s.f.adapt(np.full(s.cfg.neq, self.eps))
                w.ctx.synchronize()
                s.f.destroy()

    def close(self):
        for ws in self.workers.values():
            for w in ws:
                w.ctx.close()

    def run(self, requests, realtime: bool = True):
        """Serve the stream; returns per-request records and totals. Every
        context is served by its own host thread."""
        t0 = time.perf_counter()
        out = {}
        errors = []
        shared = {}
        for dim in self.workers:
            shared[dim] = {"pending": sorted([r for r in requests if r.dim == dim], key=lambda r: r.arrival),
                           "queue": [], "lock": threading.Lock()}
            for r in shared[dim]["pending"]:
                if self._need(dim, r) > self.capacity[dim]:
                    raise ValueError(f"request {r.rid} ({self._need(dim, r)} blocks at its peak) exceeds the "
                                     f"{dim}-D arena")

        def worker(dim, k):
            try:
                out[(dim, k)] = self._serve(dim, k, shared[dim], t0, realtime)
            except BaseException as e:   # re-raised below
                errors.append(e)
                with shared[dim]["lock"]:
                    shared[dim]["pending"].clear()
                    shared[dim]["queue"].clear()

        ths = [threading.Thread(target=worker, args=(dim, k), name=f"serve-{dim}d-{k}")
               for dim in (3, 2) for k in range(len(self.workers[dim]))]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        if errors:
            raise errors[0]
        wall = time.perf_counter() - t0
        records = {}
        total_points = 0
        phase = {}
        for (dim, k), (rec, pts, ph) in sorted(out.items()):
            records.update(rec)
            total_points += pts
            for key, v in ph.items():
                phase[f"{key}_{dim}d"] = phase.get(f"{key}_{dim}d", 0.0) + v
        tts = np.array([r["tts"] for r in records.values()]) if records else np.zeros(1)
        summary = {"requests": len(records), "wall_s": wall, "point_updates": total_points,
                   "throughput": total_points / wall,
                   "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
                   "phase_s": phase, "workers": {d: [w.capacity for w in ws] for d, ws in self.workers.items()}}
        return records, summary

    def _take(self, dim, w, sh, used, t0, realtime):
        """The waiting requests this worker admits now (earliest first)."""
        with sh["lock"]:
            now = float("inf") if not realtime else time.perf_counter() - t0
            while sh["pending"] and sh["pending"][0].arrival <= now:
                sh["queue"].append(sh["pending"].pop(0))
            others = [x for x in self.workers[dim] if x is not w]
            small = max((x.capacity for x in others), default=0)
            big_waiting = w.capacity > small and any(self._need(dim, r) > small for r in sh["queue"])
            taken = []
            for r in list(sh["queue"]):
                need = self._need(dim, r)
                if used + need > w.capacity:
                    continue
                if big_waiting and need <= small:
                    continue
                sh["queue"].remove(r)
                taken.append(r)
                used += need
            idle_until = sh["pending"][0].arrival if sh["pending"] else None
            done = not sh["pending"] and not sh["queue"]
        return taken, idle_until, done

    def _serve(self, dim, k, sh, t0, realtime):
        """The scheduling loop of one context (its own thread)."""
        w = self.workers[dim][k]
        ctx = w.ctx
        active = []
        used = 0
        records = {}
        total_points = 0
        phase = {"admit": 0.0, "refine": 0.0, "run": 0.0, "retire": 0.0}
        while True:
            ta = time.perf_counter()
            taken, idle_until, done = self._take(dim, w, sh, used, t0, realtime)
            for r in taken:
                s = Solve(r, ctx, self.base[dim])
                s.admitted = time.perf_counter() - t0
                used += s.nblk
                active.append(s)
            phase["admit"] += time.perf_counter() - ta
            if not active:
                if done:
                    break
                wait = 0.01 if idle_until is None else idle_until - (time.perf_counter() - t0)
                time.sleep(max(0.0, min(0.05, wait)))
                continue
            # one scheduling round: every active solve advances one chunk
            # (with adaptation: the solves whose cycle fits into the arena)
            group = active
            tr = time.perf_counter()
            if self.adapt:
                group, grow, mothers = [], 0, 0
                for s in active:
                    refined, m = s.cycle_need()
                    if used + grow + (refined - s.nblk) + max(mothers, m) <= w.capacity:
                        grow += refined - s.nblk
                        mothers = max(mothers, m)
                        s.cycle()
                        group.append(s)
                used += grow
                if not group:
                    raise RuntimeError(f"no {dim}-D solve fits its adaptation cycle into the arena")
            kk = min(self.chunk, min(s.req.nsteps - s.done for s in group))
            t1 = time.perf_counter()
            phase["refine"] += t1 - tr
            ctx.run([s.f for s in group], kk, use_graph=True)
            for s in group:
                s.done += kk
                total_points += s.points * kk
            if self.adapt:
                # each adaptation waits for the batched steps on the stream
                for s in group:
                    before = s.nblk
                    s.nblk = s.f.adapt(np.full(s.cfg.neq, self.eps))
                    used += s.nblk - before
            else:
                ctx.synchronize()
            t2 = time.perf_counter()
            phase["run"] += t2 - t1   # the chunk's steps and the adaptations that follow them
            tt = time.perf_counter()
            keep = []
            for s in active:
                if s.done < s.req.nsteps:
                    keep.append(s)
                    continue
                shape = (s.nblk,) + s.f.interior_shape
                flat = w.result_buffer(int(np.prod(shape)))
                u = s.f.download_interior(out=flat.reshape(shape))
                t_done = time.perf_counter() - t0
                rec = {"rid": s.req.rid, "dim": dim, "blocks": s.nblk, "arrival": s.req.arrival,
                       "admitted": s.admitted, "done": t_done, "worker": k,
                       "tts": t_done - (s.req.arrival if realtime else 0.0),
                       "time": s.f.time()[0], "checksum": float(np.dot(flat, flat))}
                if self.keep:
                    rec["u"] = u.copy()
                records[s.req.rid] = rec
                s.f.destroy()
                used -= s.nblk
            active = keep
            phase["retire"] += time.perf_counter() - tt
        return records, total_points, phase


def solve_alone(req: Request, chunk: int = 5, adapt_every: int = 0, eps: float = 1e-3, max_blocks: int = 0):
    """The same request on its own context, in the same step chunks (and,
    with adapt_every, the same adaptation cycles)."""
    base = geometry(req.dim)
    lv, _ = request_grid(req.dim, req.size)
    ctx = Context(base, max_blocks or (len(lv) * (10 if adapt_every else 1) + 64))
    if adapt_every:
        chunk = adapt_every
    try:
        s = Solve(req, ctx, base)
        while s.done < req.nsteps:
            if adapt_every:
                s.cycle()
            k = min(chunk, req.nsteps - s.done)
            ctx.run([s.f], k, use_graph=True)
            s.done += k
            if adapt_every:
                s.nblk = s.f.adapt(np.full(s.cfg.neq, eps))
        ctx.synchronize()
        return s.f.download_interior(), s.f.time()[0]
    finally:
        ctx.close()
