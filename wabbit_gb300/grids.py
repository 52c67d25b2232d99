"""Block-grid generators for tests and benchmark workloads.

A grid is a list of leaf blocks (level, integer coords) on the periodic unit
tree: level J has 2^J blocks per direction. Every generator returns a
complete, non-overlapping, 2:1-graded leaf set (gradedness across faces,
edges and corners, as ensureGradedness_tree enforces,
LIB/MESH/ensureGradedness_tree.f90:13) sorted by (level, z, y, x).
"""
from __future__ import annotations

import itertools

import numpy as np


def equidistant(dim: int, level: int):
    n = 1 << level
    if dim == 2:
        xs, ys = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
        c = np.stack([xs.ravel(), ys.ravel(), np.zeros(n * n, int)], 1)
    else:
        zs, ys, xs = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        c = np.stack([xs.ravel(), ys.ravel(), zs.ravel()], 1)
    return _sorted(np.full(len(c), level, np.int32), c.astype(np.int32))


def _sorted(level, coords):
    order = np.lexsort((coords[:, 0], coords[:, 1], coords[:, 2], level))
    return level[order].astype(np.int32), coords[order].astype(np.int32)


def _dirs(dim):
    r = [-1, 0, 1]
    for d in itertools.product(r, r, r if dim == 3 else [0]):
        if any(d):
            yield d


def balance(leaves: set, dim: int, jmin: int):
    """Refine coarse leaves until every leaf's neighbours differ by <= 1 level."""
    changed = True
    while changed:
        changed = False
        for (l, x, y, z) in sorted(leaves, key=lambda t: -t[0]):
            if (l, x, y, z) not in leaves:
                continue
            n = 1 << l
            for d in _dirs(dim):
                a = ((x + d[0]) % n, (y + d[1]) % n, (z + d[2]) % n if dim == 3 else 0)
                for lc in range(jmin, l - 1):
                    s = l - lc
                    anc = (lc, a[0] >> s, a[1] >> s, a[2] >> s if dim == 3 else 0)
                    if anc in leaves:
                        leaves.discard(anc)
                        for k in range(1 << dim):
                            leaves.add((lc + 1, 2 * anc[1] + (k >> 1 & 1), 2 * anc[2] + (k & 1),
                                        2 * anc[3] + (k >> 2 & 1) if dim == 3 else 0))
                        changed = True
                        break
    return leaves


def _to_arrays(leaves):
    arr = np.array(sorted(leaves), np.int32).reshape(-1, 4)
    return _sorted(arr[:, 0], arr[:, 1:4])


def random_graded(dim: int, jmin: int, jmax: int, seed: int, frac: float = 0.3):
    """Equidistant grid on jmin, random refinement up to jmax, then balanced."""
    rng = np.random.default_rng(seed)
    lv, co = equidistant(dim, jmin)
    leaves = {(int(l), int(c[0]), int(c[1]), int(c[2])) for l, c in zip(lv, co)}
    for _ in range(jmax - jmin):
        cand = [t for t in leaves if t[0] < jmax]
        pick = [cand[i] for i in rng.permutation(len(cand))[: max(1, int(frac * len(cand)))]]
        for (l, x, y, z) in pick:
            leaves.discard((l, x, y, z))
            for k in range(1 << dim):
                leaves.add((l + 1, 2 * x + (k >> 1 & 1), 2 * y + (k & 1), 2 * z + (k >> 2 & 1) if dim == 3 else 0))
        leaves = balance(leaves, dim, jmin)
    return _to_arrays(leaves)


def refined_around(dim: int, jmin: int, jmax: int, domain, center, radius_of_level):
    """Refine every block that intersects a ball around `center` whose radius
    depends on the level (radius_of_level(level) -> r), then balance."""
    domain = np.asarray(domain, float)[:dim]
    center = np.asarray(center, float)[:dim]
    lv, co = equidistant(dim, jmin)
    leaves = {(int(l), int(c[0]), int(c[1]), int(c[2])) for l, c in zip(lv, co)}
    for level in range(jmin, jmax):
        r = radius_of_level(level)
        h = domain / (1 << level)
        new = set()
        for (l, x, y, z) in leaves:
            if l != level:
                new.add((l, x, y, z))
                continue
            lo = np.array([x, y, z][:dim]) * h
            hi = lo + h
            # periodic distance from the ball centre to the box
            dist2 = 0.0
            for k in range(dim):
                best = np.inf
                for shift in (-domain[k], 0.0, domain[k]):
                    c = center[k] + shift
                    dk = max(lo[k] - c, 0.0, c - hi[k])
                    best = min(best, dk)
                dist2 += best * best
            if dist2 <= r * r:
                for k in range(1 << dim):
                    new.add((l + 1, 2 * x + (k >> 1 & 1), 2 * y + (k & 1), 2 * z + (k >> 2 & 1) if dim == 3 else 0))
            else:
                new.add((l, x, y, z))
        leaves = balance(new, dim, jmin)
    return _to_arrays(leaves)


def block_geometry(level, coords, domain, Bs, dim):
    """Origin x0 and spacing dx of every block (get_block_spacing_origin_b,
    LIB/TREE/module_treelib.f90:96-101)."""
    level = np.asarray(level)
    dx = np.zeros((len(level), 3))
    x0 = np.zeros((len(level), 3))
    for d in range(dim):
        dx[:, d] = 2.0 ** (-level.astype(float)) * domain[d] / Bs[d]
        x0[:, d] = (np.asarray(coords)[:, d] * Bs[d]).astype(float) * dx[:, d]
    return x0, dx
