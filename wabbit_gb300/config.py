"""Run configuration: the ctypes mirror of ``wg_config`` (include/wabbit_gb300.h)
and a reader for the reference's .ini files.

The .ini format is WABBIT's ``key=value;`` lines inside ``[Section]`` headers
(LIB/PARAMS/module_ini_files_parser_mpi.f90). Only the keys that the hot path
reads are interpreted; their defaults follow the reference
(LIB/MESH/ini_file_to_params.f90:2-647, LIB/EQUATION/ACMnew/module_ACM.f90:
172-609). Unknown keys are ignored, as in the reference.
"""
from __future__ import annotations

import ctypes
import re


class WgConfig(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("Bs", ctypes.c_int * 3),
        ("g", ctypes.c_int),
        ("g_rhs", ctypes.c_int),
        ("neq", ctypes.c_int),
        ("domain", ctypes.c_double * 3),
        ("Jmin", ctypes.c_int),
        ("Jmax", ctypes.c_int),
        ("wavelet", ctypes.c_char * 16),
        ("c0", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("gamma_p", ctypes.c_double),
        ("skew_symmetry", ctypes.c_int),
        ("penalization", ctypes.c_int),
        ("C_eta", ctypes.c_double),
        ("use_sponge", ctypes.c_int),
        ("C_sponge", ctypes.c_double),
        ("u_mean_set", ctypes.c_double * 3),
        ("CFL", ctypes.c_double),
        ("CFL_nu", ctypes.c_double),
        ("CFL_eta", ctypes.c_double),
        ("dt_fixed", ctypes.c_double),
        ("dt_max", ctypes.c_double),
        ("time_max", ctypes.c_double),
        ("write_time", ctypes.c_double),
        ("tsave_stats", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("eps_normalized", ctypes.c_int),
        ("threshold_state_vector_component", ctypes.c_int * 8),
        ("rhs_precision", ctypes.c_int),
        ("threshold_mask", ctypes.c_int),
        ("force_maxlevel_dealiasing", ctypes.c_int),
        ("use_coarse_extension", ctypes.c_int),
        ("reserved", ctypes.c_int * 11),
    ]

    def copy(self) -> "WgConfig":
        c = WgConfig()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(WgConfig))
        return c

    @property
    def nx(self) -> int:
        return self.Bs[0] + 2 * self.g

    @property
    def nz(self) -> int:
        return self.Bs[2] + 2 * self.g if self.dim == 3 else 1

    @property
    def npts(self) -> int:
        return self.nx * (self.Bs[1] + 2 * self.g) * self.nz


class WgGeometry(ctypes.Structure):
    """ctypes mirror of ``wg_geometry`` (the penalisation geometry a tree's
    masks are drawn from)."""
    _fields_ = [
        ("kind", ctypes.c_int),
        ("sponge_type", ctypes.c_int),
        ("x_cntr", ctypes.c_double * 3),
        ("R_cyl", ctypes.c_double),
        ("C_smooth", ctypes.c_double),
        ("L_sponge", ctypes.c_double),
        ("p_sponge", ctypes.c_double),
        ("reserved", ctypes.c_int * 8),
    ]


GEOM_NONE, GEOM_CYLINDER, GEOM_SPHERE = 0, 1, 2
SPONGE_RECT, SPONGE_PNORM = 0, 1


# wavelet -> default number of ghost nodes g and the RHS ghost width g_rhs
# (setup_wavelet, module_wavelets.f90:1327-1340; ini_file_to_params.f90:293-310
# raises both to the FD_4th_central stencil half-width 2)
def wavelet_ghosts(wavelet: str) -> tuple[int, int]:
    X, Y = int(wavelet[3]), int(wavelet[4])
    hr = X - 1                       # HR support -(X-1)..(X-1)
    hd = 0 if Y == 0 else (X - 1) + (Y - 1)
    g = max(hr, hd, 2)
    g_rhs = max(X // 2, 2)
    return g, g_rhs


def defaults(dim: int = 2) -> WgConfig:
    """Reference defaults for an ACM run with FD_4th_central."""
    c = WgConfig()
    c.dim = dim
    c.Bs[:] = (17, 17, 17 if dim == 3 else 1)
    c.wavelet = b"CDF40"
    g_min, g_rhs = wavelet_ghosts("CDF40")
    c.g, c.g_rhs = g_min, g_rhs
    c.neq = dim + 1
    c.domain[:] = (1.0, 1.0, 1.0)
    c.Jmin, c.Jmax = 1, 1
    c.c0, c.nu, c.gamma_p = 10.0, 1e-1, 1.0
    c.skew_symmetry = 0
    c.penalization, c.C_eta = 1, 1.0
    c.use_sponge, c.C_sponge = 0, 1e-2
    c.u_mean_set[:] = (1.0, 0.0, 0.0)
    c.CFL, c.CFL_eta = 1.0, 0.99
    # FD4: CFL_nu = 0.95*2.79/(5.333*dim) (module_ACM.f90:370-376)
    c.CFL_nu = 0.95 * 2.79 / (5.333 * float(dim))
    c.dt_fixed, c.dt_max = 0.0, 0.0
    c.time_max = 1.0
    c.write_time = 0.0
    c.tsave_stats = 0.0
    c.eps, c.eps_normalized = 1e-3, 0
    for i in range(8):
        c.threshold_state_vector_component[i] = 1
    c.rhs_precision = 0
    return c


def _parse_ini(text: str) -> dict:
    sec = None
    out: dict = {}
    for raw in text.splitlines():
        line = raw.split(";")[0].split("!")[0].strip() if not raw.strip().startswith(";") else ""
        if not line or line.startswith("#") or line.startswith("%"):
            continue
        m = re.match(r"^\[(.+)\]$", line)
        if m:
            sec = m.group(1).strip()
            continue
        if "=" in line and sec is not None:
            k, v = line.split("=", 1)
            out[(sec, k.strip())] = v.strip()
    return out


def _num(v: str) -> list[float]:
    return [float(x) for x in v.replace(",", " ").split()]


def from_ini(path: str) -> WgConfig:
    """Read the hot-path keys of a WABBIT .ini file into a WgConfig."""
    with open(path, errors="ignore") as f:
        return from_ini_text(f.read())


def from_ini_text(text: str) -> WgConfig:
    """The hot-path keys of a WABBIT .ini file's text as a WgConfig."""
    kv = _parse_ini(text)

    def get(sec, key, default=None):
        v = kv.get((sec, key), "")
        return default if v == "" else v

    dim = int(get("Domain", "dim", "2"))
    c = defaults(dim)
    dom = get("Domain", "domain_size")
    if dom:
        d = _num(dom)
        for i in range(dim):
            c.domain[i] = d[i]
    wav = get("Wavelet", "wavelet", "CDF40")
    c.wavelet = wav.encode()
    g_min, g_rhs = wavelet_ghosts(wav)
    c.g = int(get("Blocks", "number_ghost_nodes", g_min))
    c.g_rhs = max(int(get("Blocks", "number_ghost_nodes_rhs", g_rhs)), g_rhs)
    bs = get("Blocks", "number_block_nodes")
    if bs:
        b = [int(x) for x in _num(bs)]
        b = b * dim if len(b) == 1 else b
        for i in range(dim):
            c.Bs[i] = b[i]
    c.neq = int(get("Blocks", "number_equations", dim + 1))
    c.Jmax = int(get("Blocks", "max_treelevel", 1))
    c.Jmin = int(get("Blocks", "min_treelevel", 1))
    c.eps = float(get("Blocks", "eps", 1e-3))
    c.eps_normalized = int(float(get("Blocks", "eps_normalized", 0)))
    tsv = get("Blocks", "threshold_state_vector_component")
    if tsv:
        for i, v in enumerate(_num(tsv)):
            c.threshold_state_vector_component[i] = int(v)
    c.c0 = float(get("ACM-new", "c_0", 10.0))
    c.nu = float(get("ACM-new", "nu", 1e-1))
    c.gamma_p = float(get("ACM-new", "gamma_p", 1.0))
    c.skew_symmetry = int(float(get("ACM-new", "skew_symmetry", 0)))
    ums = get("ACM-new", "u_mean_set")
    if ums:
        for i, v in enumerate(_num(ums)[:3]):
            c.u_mean_set[i] = v
    c.penalization = int(float(get("VPM", "penalization", 1)))
    c.C_eta = float(get("VPM", "C_eta", 1.0))
    c.use_sponge = int(float(get("Sponge", "use_sponge", 0)))
    c.C_sponge = float(get("Sponge", "C_sponge", 1e-2))
    c.CFL = float(get("Time", "CFL", 1.0))
    c.CFL_eta = float(get("Time", "CFL_eta", 0.99))
    c.CFL_nu = float(get("Time", "CFL_nu", 0.95 * 2.79 / (5.333 * float(dim))))
    c.dt_fixed = float(get("Time", "dt_fixed", 0.0))
    c.dt_max = float(get("Time", "dt_max", 0.0))
    c.time_max = float(get("Time", "time_max", 1.0))
    if get("Time", "write_method", "fixed_freq") == "fixed_time":
        c.write_time = float(get("Time", "write_time", 1.0))
    ts = get("Statistics", "tsave_stats")
    c.tsave_stats = float(ts) if ts else 0.0
    c.threshold_mask = int(float(get("Blocks", "threshold_mask", 0)))
    c.force_maxlevel_dealiasing = int(float(get("Blocks", "force_maxlevel_dealiasing", 0)))
    # useCoarseExtension / useSecurityZone: on by default for lifted wavelets
    # only (ini_file_to_params.f90:543-546); either set for an unlifted one
    # switches the coarse-extension path on
    ce = get("Blocks", "useCoarseExtension")
    sz = get("Blocks", "useSecurityZone")
    c.use_coarse_extension = int(any(v is not None and str(v).strip() not in ("", "0") for v in (ce, sz)))
    return c


def geometry_from_ini(path: str, cfg: WgConfig | None = None) -> WgGeometry:
    """The penalisation geometry of a WABBIT .ini file ([VPM] geometry,
    x_cntr, R_cyl, C_smooth; [Sponge] sponge_type, L_sponge, p_sponge) with
    the reference's defaults (module_ACM.f90:290-362)."""
    with open(path, errors="ignore") as f:
        return geometry_from_ini_text(f.read(), cfg)


def geometry_from_ini_text(text: str, cfg: WgConfig | None = None) -> WgGeometry:
    """geometry_from_ini on the text of an .ini file."""
    kv = _parse_ini(text)

    def get(sec, key, default=None):
        v = kv.get((sec, key), "")
        return default if v == "" else v

    cfg = cfg or from_ini_text(text)
    geo = WgGeometry()
    name = get("VPM", "geometry", "none").lower().replace("_", "")
    kinds = {"cylinder": GEOM_CYLINDER, "circle": GEOM_CYLINDER, "sphere-fixed": GEOM_SPHERE, "none": GEOM_NONE}
    if name not in kinds:
        raise ValueError(f"geometry {name!r} is not supported")
    geo.kind = kinds[name]
    xc = get("VPM", "x_cntr")
    xs = _num(xc) if xc else [0.5 * cfg.domain[i] for i in range(3)]
    for i in range(3):
        geo.x_cntr[i] = xs[i] if i < len(xs) else 0.5 * cfg.domain[i]
    geo.R_cyl = float(get("VPM", "R_cyl", 0.5))
    geo.C_smooth = float(get("VPM", "C_smooth", 1.5))
    st = get("Sponge", "sponge_type", "rect")
    if st not in ("rect", "p-norm"):
        raise ValueError(f"sponge_type {st!r} is not supported")
    geo.sponge_type = SPONGE_PNORM if st == "p-norm" else SPONGE_RECT
    geo.L_sponge = float(get("Sponge", "L_sponge", 0.0))
    geo.p_sponge = float(get("Sponge", "p_sponge", 20.0))
    return geo
