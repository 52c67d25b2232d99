"""Shared helpers of the test suite (no GPU needed)."""
import numpy as np

from wabbit_gb300 import config, grids


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def small_cfg(dim, wavelet="CDF40", g=None, Bs=8, jmin=1, jmax=4, skew=0, penal=0):
    c = config.defaults(dim)
    for d in range(dim):
        c.Bs[d] = Bs
    c.wavelet = wavelet.encode()
    g_min, g_rhs = config.wavelet_ghosts(wavelet)
    c.g = g if g is not None else g_min
    c.g_rhs = g_rhs
    c.Jmin, c.Jmax = jmin, jmax
    c.domain[:] = (1.0, 1.25, 1.5)
    c.c0, c.nu, c.gamma_p = 10.0, 1e-2, 1.0
    c.skew_symmetry, c.penalization = skew, penal
    c.CFL = 0.5
    c.time_max = 1e9
    return c


def smooth_state(cfg, lv, co, seed):
    """A smooth periodic field evaluated on every point incl. ghosts."""
    rng = np.random.default_rng(seed)
    dim = cfg.dim
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, dim)
    g = cfg.g
    nb = len(lv)
    out = np.zeros((nb, cfg.neq, cfg.nz, cfg.Bs[1] + 2 * g, cfg.nx))
    ix = np.arange(cfg.nx) - g
    iy = np.arange(cfg.Bs[1] + 2 * g) - g
    iz = np.arange(cfg.nz) - (g if dim == 3 else 0)
    for c in range(cfg.neq):
        k = rng.integers(1, 3, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        amp = rng.uniform(0.2, 1.0)
        for b in range(nb):
            X = x0[b, 0] + ix * dx[b, 0]
            Y = x0[b, 1] + iy * dx[b, 1]
            Z = x0[b, 2] + iz * dx[b, 2] if dim == 3 else np.zeros(1)
            f = (np.sin(2 * np.pi * k[0] * X / cfg.domain[0] + ph[0])[None, None, :]
                 * np.cos(2 * np.pi * k[1] * Y / cfg.domain[1] + ph[1])[None, :, None]
                 * (np.cos(2 * np.pi * k[2] * Z / cfg.domain[2] + ph[2])[:, None, None] if dim == 3 else 1.0))
            out[b, c] = amp * f + (0.5 if c == 0 else 0.0)
    return out


def random_state(cfg, nb, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nb, cfg.neq, cfg.nz, cfg.Bs[1] + 2 * cfg.g, cfg.nx))


def sphere_mask(cfg, lv, co, center, radius):
    """chi = smoothed step of the distance to a sphere, colour 1, u_s = 0."""
    x0, dx = grids.block_geometry(lv, co, cfg.domain, cfg.Bs, cfg.dim)
    g = cfg.g
    nb = len(lv)
    m = np.zeros((nb, 6, cfg.nz, cfg.Bs[1] + 2 * g, cfg.nx))
    ix = np.arange(cfg.nx) - g
    iy = np.arange(cfg.Bs[1] + 2 * g) - g
    iz = np.arange(cfg.nz) - (g if cfg.dim == 3 else 0)
    h = 1.5 * min(cfg.domain[d] / cfg.Bs[d] / 2 ** cfg.Jmax for d in range(cfg.dim))
    for b in range(nb):
        X = (x0[b, 0] + ix * dx[b, 0])[None, None, :]
        Y = (x0[b, 1] + iy * dx[b, 1])[None, :, None]
        Z = (x0[b, 2] + iz * dx[b, 2])[:, None, None] if cfg.dim == 3 else 0.0
        r = np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2 + ((Z - center[2]) ** 2 if cfg.dim == 3 else 0))
        chi = np.clip(0.5 * (1 - np.cos(np.pi * (radius + h - r) / (2 * h))), 0, 1)
        chi = np.where(r < radius - h, 1.0, np.where(r > radius + h, 0.0, chi))
        m[b, 0] = chi
        m[b, 4] = np.where(chi > 0, 1.0, 0.0)
        m[b, 5] = 0.0
    return m


def vortex_cfg():
    c = config.defaults(2)
    c.Bs[0] = c.Bs[1] = 32
    c.domain[0] = c.domain[1] = 6.283185307179586
    c.wavelet = b"CDF40"
    c.g, c.g_rhs = 3, 2
    c.Jmin = c.Jmax = 3
    c.c0, c.nu, c.gamma_p = 7.0, 5.0e-5, 1.0
    c.skew_symmetry, c.penalization = 1, 0
    c.CFL = 1.0
    c.time_max, c.write_time = 20.0, 10.0
    return c


