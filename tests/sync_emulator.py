"""NumPy emulation of the device ghost-sync kernel (k_sync.cu) driven by the
host patch table (wg_sync_table_host). Lets the CPU suite check the table
generator against the oracle without a GPU."""
import ctypes

import numpy as np

from wabbit_gb300 import capi

PRED = {2: [0.5, 0.5], 4: [c / 16.0 for c in (-1.0, 9.0, 9.0, -1.0)],
        6: [c / 256.0 for c in (3.0, -25.0, 150.0, 150.0, -25.0, 3.0)],
        8: [c / 2048.0 for c in (-5.0, 49.0, -245.0, 1225.0, 1225.0, -245.0, 49.0, -5.0)]}


def host_table(cfg, level, coords, gm, gp, thin=False):
    L = capi.load()
    level = np.ascontiguousarray(level, np.int32)
    coords = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
    ip = ctypes.POINTER(ctypes.c_int)
    n = capi.check(L.wg_sync_table_host(ctypes.byref(cfg), len(level), level.ctypes.data_as(ip),
                                        coords.ctypes.data_as(ip), gm, gp, 1 if thin else 0, 0, None))
    out = np.zeros((n, 19), np.int32)
    capi.check(L.wg_sync_table_host(ctypes.byref(cfg), len(level), level.ctypes.data_as(ip),
                                    coords.ctypes.data_as(ip), gm, gp, 1 if thin else 0, n, out.ctypes.data_as(ip)))
    return out


def _pred_value(coarse, f, order):
    """Value of the reference's fine array at fine index f (z, y, x order)."""
    c = PRED[order]
    h = order - 1

    def vx(fz, fy, fx):
        if fx % 2 == 0:
            return coarse[fz // 2, fy // 2, fx // 2]
        if fx < h or fx > 2 * coarse.shape[2] - 2 - h:
            return 0.0
        s = c[0] * coarse[fz // 2, fy // 2, (fx - h) // 2]
        for m in range(1, order):
            s = s + c[m] * coarse[fz // 2, fy // 2, (fx - h + 2 * m) // 2]
        return s

    def vxy(fz, fy, fx):
        if fy % 2 == 0:
            return vx(fz, fy, fx)
        if fy < h or fy > 2 * coarse.shape[1] - 2 - h:
            return 0.0
        s = c[0] * vx(fz, fy - h, fx)
        for m in range(1, order):
            s = s + c[m] * vx(fz, fy - h + 2 * m, fx)
        return s

    fz, fy, fx = f
    if fz % 2 == 0:
        return vxy(fz, fy, fx)
    if fz < h or fz > 2 * coarse.shape[0] - 2 - h:
        return 0.0
    s = c[0] * vxy(fz - h, fy, fx)
    for m in range(1, order):
        s = s + c[m] * vxy(fz - h + 2 * m, fy, fx)
    return s


def apply(table, data, order):
    """Apply the patches stage by stage to data (nb, nc, nz, ny, nx) in place."""
    for stage in sorted(set(table[:, 3])):
        for p in table[table[:, 3] == stage]:
            src, dst, op = p[0], p[1], p[2]
            rlo, rhi, slo, shi, blo = p[4:7], p[7:10], p[10:13], p[13:16], p[16:19]
            for iz in range(rhi[2] - rlo[2] + 1):
                for iy in range(rhi[1] - rlo[1] + 1):
                    for ix in range(rhi[0] - rlo[0] + 1):
                        d = (rlo[2] + iz, rlo[1] + iy, rlo[0] + ix)
                        if op == 0:
                            s = (slo[2] + iz, slo[1] + iy, slo[0] + ix)
                            data[dst, :, d[0], d[1], d[2]] = data[src, :, s[0], s[1], s[2]]
                        elif op == 1:
                            s = (slo[2] + 2 * (blo[2] + iz), slo[1] + 2 * (blo[1] + iy), slo[0] + 2 * (blo[0] + ix))
                            data[dst, :, d[0], d[1], d[2]] = data[src, :, s[0], s[1], s[2]]
                        else:
                            f = (blo[2] + iz, blo[1] + iy, blo[0] + ix)
                            for c in range(data.shape[1]):
                                coarse = data[src, c, slo[2]:shi[2] + 1, slo[1]:shi[1] + 1, slo[0]:shi[0] + 1]
                                data[dst, c, d[0], d[1], d[2]] = _pred_value(coarse, f, order)
    return data
