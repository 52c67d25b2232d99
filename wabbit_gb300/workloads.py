"""Synthetic workloads of the ACM hot path (seeded, reproducible).

The reference publishes no benchmark inputs; these generators build the
grids, initial conditions and penalisation masks of the run configurations
the measurements are quoted on:

* ``acm2d_vortex``  -- 2-D ACM on periodic [0,1]^2, Bs=16, g=4, CDF4,0,
  Jmin=2, Jmax=5, nu=1e-3, c0=20, CFL=0.5, no mask; IC: sum of 8 Gaussian
  velocity vortices (centres U[0,1)^2, radius U[0.03,0.08], circulation N(0,1),
  seed 1), p = 0. Grid: refined to Jmax around the vortex centres.
* ``acm3d_sphere``  -- 3-D ACM with volume penalisation on [0,4]x[0,2]x[0,2],
  Bs=16^3, g=6 (CDF4,4 needs g >= 6), Jmax=6, C_eta=1e-3, nu=1e-3, c0=15,
  CFL=0.5; sphere of radius 0.2 at the domain centre with the reference's
  cosine-smoothed mask (C_smooth = 1.5 dx_min); IC: u = (1,0,0) + 0.01 N(0,1)
  per point and component (seed 2), p = 0. Grid: refined around the sphere
  with level-dependent radii (about 4k blocks at Jmax=6).
* ``acm3d_sphere_j7`` -- the same physics at Jmax=7 with the stencils and
  the stage arithmetic evaluated in double-float arithmetic on the FP32 units
  (FP64 state); grid refined around the sphere with wider level-dependent
  radii (36,688 blocks over levels 3-7).

* ``adapt3d_cdf44`` -- the adapt path at scale: 3-D, Bs=16^3, g=6, CDF4,4,
  periodic [0,1]^3, 99,184 blocks over levels 3-7 (four level jumps),
  threshold eps=1e-4 (Linfty-normalised). Field (seed 5), per component: 16
  Fourier modes with integer wave vectors |k| <= 8 drawn uniformly, random
  phases and N(0,1)/|k|^2 amplitudes, plus 32 fronts tanh((n.x - d)/0.01)
  with uniformly random unit normals n and offsets d (minimum image on the
  torus); evaluated on the device (`adapt_field_device`).

All random draws use numpy's PCG64 generator with the stated seed, in block
order, component order, then point order (x fastest).
"""
from __future__ import annotations

import numpy as np

from . import config, grids

WORKLOADS = ("acm2d_vortex", "acm3d_sphere", "acm3d_sphere_j7", "adapt3d_cdf44")


def make_config(name: str):
    if name == "acm2d_vortex":
        c = config.defaults(2)
        c.Bs[0] = c.Bs[1] = 16
        c.domain[0] = c.domain[1] = 1.0
        c.wavelet = b"CDF40"
        c.g, c.g_rhs = 4, 2
        c.Jmin, c.Jmax = 2, 5
        c.nu, c.c0, c.gamma_p = 1e-3, 20.0, 1.0
        c.penalization = 0
        c.CFL = 0.5
        c.eps, c.eps_normalized = 1e-3, 0
        c.time_max = 1e9
        return c
    if name in ("acm3d_sphere", "acm3d_sphere_j7"):
        c = config.defaults(3)
        c.Bs[:] = (16, 16, 16)
        c.domain[:] = (4.0, 2.0, 2.0)
        c.wavelet = b"CDF44"
        c.g, c.g_rhs = 6, 2
        c.Jmin = 2
        c.Jmax = 7 if name.endswith("j7") else 6
        # config 3: FP32-pipe stencils (double-float) with FP64 RK state
        c.rhs_precision = 1 if name.endswith("j7") else 0
        c.nu, c.c0, c.gamma_p = 1e-3, 15.0, 1.0
        c.penalization, c.C_eta = 1, 1e-3
        c.CFL = 0.5
        c.eps, c.eps_normalized = 1e-3, 1
        c.u_mean_set[:] = (1.0, 0.0, 0.0)
        c.time_max = 1e9
        return c
    if name == "adapt3d_cdf44":
        c = config.defaults(3)
        c.Bs[:] = (16, 16, 16)
        c.domain[:] = (1.0, 1.0, 1.0)
        c.wavelet = b"CDF44"
        c.g, c.g_rhs = 6, 2
        c.Jmin, c.Jmax = 3, 7
        c.eps, c.eps_normalized = 1e-4, 1
        c.penalization = 0
        c.time_max = 1e9
        return c
    raise ValueError(f"unknown workload {name}")


def make_grid(name: str, cfg):
    if name == "acm2d_vortex":
        rng = np.random.default_rng(1)
        centres = rng.uniform(0.0, 1.0, size=(8, 2))
        leaves = None
        lv_all, co_all = None, None
        # refine around every vortex centre
        from .grids import balance, equidistant, _to_arrays
        lv, co = equidistant(2, cfg.Jmin)
        leaves = {(int(l), int(c[0]), int(c[1]), 0) for l, c in zip(lv, co)}
        for level in range(cfg.Jmin, cfg.Jmax):
            r = 0.06 + 0.25 * 2.0 ** (-(level - cfg.Jmin))
            h = 1.0 / (1 << level)
            new = set()
            for (l, x, y, z) in leaves:
                hit = False
                if l == level:
                    for cx, cy in centres:
                        dx = min(abs((x + 0.5) * h - cx), 1 - abs((x + 0.5) * h - cx))
                        dy = min(abs((y + 0.5) * h - cy), 1 - abs((y + 0.5) * h - cy))
                        if max(dx, dy) < r + 0.5 * h:
                            hit = True
                            break
                if hit:
                    for k in range(4):
                        new.add((l + 1, 2 * x + (k >> 1 & 1), 2 * y + (k & 1), 0))
                else:
                    new.add((l, x, y, z))
            leaves = balance(new, 2, cfg.Jmin)
        return _to_arrays(leaves)
    centre = [0.5 * cfg.domain[d] for d in range(3)]
    jmin = cfg.Jmin
    a, b = (0.3, 0.8) if name.endswith("j7") else (0.16, 0.32) if name == "adapt3d_cdf44" else (0.2, 0.6)
    return grids.refined_around(3, jmin, cfg.Jmax, cfg.domain, centre, lambda l: a + b * 2.0 ** (-(l - jmin)))


def _points(cfg, lv, co):
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, cfg.dim)
    return x0, dx


def initial_condition(name: str, cfg, lv, co):
    """Interior initial state, shape (nblk, neq, Bz, By, Bx)."""
    nb = len(lv)
    Bx, By = cfg.Bs[0], cfg.Bs[1]
    Bz = cfg.Bs[2] if cfg.dim == 3 else 1
    x0, dx = _points(cfg, lv, co)
    if name == "acm2d_vortex":
        rng = np.random.default_rng(1)
        centres = rng.uniform(0.0, 1.0, size=(8, 2))
        radius = rng.uniform(0.03, 0.08, size=8)
        gamma = rng.normal(0.0, 1.0, size=8)
        u = np.zeros((nb, 3, 1, By, Bx))
        ix = np.arange(Bx)
        iy = np.arange(By)
        X = x0[:, 0, None, None] + ix[None, None, :] * dx[:, 0, None, None]
        Y = x0[:, 1, None, None] + iy[None, :, None] * dx[:, 1, None, None]
        for k in range(8):
            ddx = X - centres[k, 0]
            ddy = Y - centres[k, 1]
            ddx -= np.rint(ddx)          # minimum image on the unit torus
            ddy -= np.rint(ddy)
            r2 = ddx ** 2 + ddy ** 2
            amp = gamma[k] / (np.pi * radius[k] ** 2) * np.exp(-r2 / radius[k] ** 2)
            u[:, 0, 0] += -amp * ddy
            u[:, 1, 0] += amp * ddx
        return u
    rng = np.random.default_rng(2)
    u = 0.01 * rng.standard_normal((nb, 4, Bz, By, Bx))
    u[:, 0] += 1.0
    u[:, 3] = 0.0
    return u


def adapt_field_device(cfg, lv, co, seed: int = 5, nmodes: int = 16, nfronts: int = 32, chunk: int = 4096,
                       device: str = "cuda"):
    """Interior field of the adapt workload on the GPU (or `device`; torch
    float64), shape (nblk, 4, Bz, By, Bx)."""
    import torch
    rng = np.random.default_rng(seed)
    dev = torch.device(device)
    nc = cfg.neq
    params = []
    for _ in range(nc):
        ks = []
        while len(ks) < nmodes:
            k = rng.integers(-8, 9, size=3)
            if 0 < np.linalg.norm(k) <= 8:
                ks.append(k)
        ks = np.array(ks, float)
        phase = rng.uniform(0.0, 2.0 * np.pi, size=nmodes)
        amp = rng.normal(0.0, 1.0, size=nmodes) / np.sum(ks * ks, axis=1)
        n = rng.normal(size=(nfronts, 3))
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        d = rng.uniform(0.0, 1.0, size=(nfronts, 3))
        params.append((ks, phase, amp, n, d))
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, 3)
    B = cfg.Bs[0]
    out = torch.empty((len(lv), nc, B, B, B), device=dev, dtype=torch.float64)
    ar = torch.arange(B, device=dev, dtype=torch.float64)
    for s0 in range(0, len(lv), chunk):
        s1 = min(len(lv), s0 + chunk)
        X0 = torch.as_tensor(x0[s0:s1], device=dev)
        DX = torch.as_tensor(dx[s0:s1], device=dev)
        X = X0[:, 0, None, None, None] + ar[None, None, None, :] * DX[:, 0, None, None, None]
        Y = X0[:, 1, None, None, None] + ar[None, None, :, None] * DX[:, 1, None, None, None]
        Z = X0[:, 2, None, None, None] + ar[None, :, None, None] * DX[:, 2, None, None, None]
        for c, (ks, phase, amp, n, d) in enumerate(params):
            f = torch.zeros((s1 - s0, B, B, B), device=dev, dtype=torch.float64)
            for m in range(len(ks)):
                arg = 2.0 * np.pi * (ks[m, 0] * X + ks[m, 1] * Y + ks[m, 2] * Z) + phase[m]
                f += amp[m] * torch.cos(arg)
            for m in range(len(n)):
                r = [X - d[m, 0], Y - d[m, 1], Z - d[m, 2]]
                r = [q - torch.round(q) for q in r]
                f += torch.tanh((n[m, 0] * r[0] + n[m, 1] * r[1] + n[m, 2] * r[2]) / 0.01)
            out[s0:s1, c] = f
    return out


def sphere_mask(cfg, lv, co, centre=None, radius=0.2, C_smooth=1.5):
    """Mask of a fixed sphere for the blocks it touches (create_mask_3D_acm
    'sphere-fixed' -> draw_sphere, LIB/EQUATION/ACMnew/create_mask.f90:58-61,
    LIB/EQUATION/insects/module_geometry.f90:49-117, step_cosine4
    LIB/HELPER/module_helpers.f90:467-487): chi = cosine-smoothed step of the
    signed distance over the width h = C_smooth*dx_min, colour 1, u_s = 0.
    Returns (block ids, masks (n, 6, nz, ny, nx) in the hvy_mask layout)."""
    centre = np.asarray(centre if centre is not None else [0.5 * cfg.domain[d] for d in range(3)])
    dx_min = min(2.0 ** (-cfg.Jmax) * cfg.domain[d] / cfg.Bs[d] for d in range(cfg.dim))
    h = C_smooth * dx_min
    safety = h
    x0, dx = _points(cfg, lv, co)
    g = cfg.g
    ids, masks = [], []
    ny = cfg.Bs[1] + 2 * g
    for b in range(len(lv)):
        lo = x0[b] - g * dx[b]
        hi = x0[b] + (np.array(cfg.Bs) + g) * dx[b]
        d2 = sum(max(lo[k] - centre[k], 0.0, centre[k] - hi[k]) ** 2 for k in range(3))
        if np.sqrt(d2) > radius + safety + 3 * dx[b].max():
            continue
        ix = np.arange(cfg.nx) - g
        X = (x0[b, 0] + ix * dx[b, 0])[None, None, :]
        Y = (x0[b, 1] + (np.arange(ny) - g) * dx[b, 1])[None, :, None]
        Z = (x0[b, 2] + (np.arange(cfg.nz) - g) * dx[b, 2])[:, None, None]
        dist = np.sqrt((X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2) - radius
        chi = np.where(dist <= -h, 1.0, np.where(dist >= h, 0.0, 0.5 * (1.0 + np.cos((dist + h) * np.pi / (2.0 * h)))))
        if not (chi > 0).any():
            continue
        m = np.zeros((6, cfg.nz, ny, cfg.nx))
        m[0] = chi
        m[4] = 1.0
        ids.append(b)
        masks.append(m)
    if not ids:
        return np.zeros(0, np.int32), np.zeros((0, 6, cfg.nz, ny, cfg.nx))
    return np.array(ids, np.int32), np.stack(masks)


def build(name: str, jmax: int | None = None):
    """(cfg, level, coords, interior IC, mask ids, masks)."""
    cfg = make_config(name)
    if jmax is not None:
        cfg.Jmax = jmax
    lv, co = make_grid(name, cfg)
    u = initial_condition(name, cfg, lv, co)
    if cfg.dim == 3 and cfg.penalization:
        ids, masks = sphere_mask(cfg, lv, co)
    else:
        ids, masks = np.zeros(0, np.int32), None
    return cfg, lv, co, u, ids, masks
