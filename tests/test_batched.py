"""Batched stepping of several independent solves (trees) in one context:
with the FP32-pipe precision, wg_run steps all listed trees with one launch
per kernel (block lists, ghost gathers and prediction patches of all trees
concatenated). Every tree's result must be bit-identical to the same tree
stepped alone, whatever the mix, and stay within the FP32-pipe tolerance of
the FP64 oracle."""
import numpy as np
import pytest

from helpers import rel_l2, small_cfg, smooth_state, sphere_mask
from pyoracle import Oracle, interior
from wabbit_gb300 import grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _solves(dim):
    """Three solves of one block geometry with different grids, viscosity,
    time-step limits and masks."""
    out = []
    for k, (seed, nu, masked) in enumerate([(3, 1e-2, True), (7, 5e-3, False), (11, 2e-2, True)]):
        cfg = small_cfg(dim, "CDF44", Bs=16 if dim == 3 else 12, penal=1 if masked else 0,
                        jmin=1 if dim == 3 else 2, jmax=2 if dim == 3 else 4)
        cfg.C_eta = 1e-2
        cfg.nu = nu
        cfg.rhs_precision = 1
        lv, co = grids.random_graded(dim, cfg.Jmin, cfg.Jmax, seed=seed, frac=0.35)
        data = smooth_state(cfg, lv, co, 40 + k)
        mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.25) if masked else None
        out.append((cfg, lv, co, data, mask))
    return out


def _load(ctx, cfg, lv, co, data, mask):
    f = ctx.forest(cfg)
    f.set_grid(lv, co)
    f.upload(data)
    f.set_mask(mask)
    f.set_time(0.0)
    return f


@pytest.mark.parametrize("dim", [2, 3])
def test_batched_equals_alone(dim):
    solves = _solves(dim)
    cap = sum(len(s[1]) for s in solves) + 8
    nsteps = 3
    alone = []
    for s in solves:
        with Context(s[0], cap) as ctx:
            f = _load(ctx, *s)
            f.run(nsteps, use_graph=True)
            alone.append((f.download(), f.time()))
    with Context(solves[0][0], cap) as ctx:
        fs = [_load(ctx, *s) for s in solves]
        ctx.run(fs, 1, use_graph=False)        # one batched step without a graph
        ctx.run(fs, nsteps - 1, use_graph=True)
        for f, (ref, tref) in zip(fs, alone):
            assert np.array_equal(f.download(), ref)
            assert f.time() == tref
        # a different mix (two of the three) keeps each solve's result
        with Context(solves[0][0], cap) as ctx2:
            gs = [_load(ctx2, *s) for s in (solves[2], solves[0])]
            ctx2.run(gs, nsteps, use_graph=True)
            assert np.array_equal(gs[0].download(), alone[2][0])
            assert np.array_equal(gs[1].download(), alone[0][0])


def test_batched_within_tolerance_of_oracle():
    cfg, lv, co, data, mask = _solves(3)[0]
    o = Oracle(cfg)
    o.set_grid(lv, co, data)
    o.set_mask(mask)
    t = 0.0
    for _ in range(2):
        t, _ = o.step(t)
    others = _solves(3)[1:]
    with Context(cfg, sum(len(s[1]) for s in _solves(3)) + 8) as ctx:
        f = _load(ctx, cfg, lv, co, data, mask)
        gs = [_load(ctx, *s) for s in others]
        ctx.run([gs[0], f, gs[1]], 2, use_graph=True)
        assert rel_l2(interior(cfg, f.download()), interior(cfg, o.data())) < 1e-12


def test_tree_listed_twice_rejected():
    from wabbit_gb300 import capi
    cfg, lv, co, data, mask = _solves(2)[1]
    with Context(cfg, len(lv) + 4) as ctx:
        f = _load(ctx, cfg, lv, co, data, mask)
        with pytest.raises(capi.WgError):
            ctx.run([f, f], 1)


def test_batched_stage_forms_bit_identical_on_many_slabs():
    """Three 3-D solves of a few hundred 16^3 blocks each, stepped together:
    the persistent slab form (each CTA walks many slabs, crossing the trees'
    boundaries, where stage 4 hands its running maximum to the right tree)
    gives the same bits and times as the tile and direct forms."""
    solves = []
    for k, (seed, nu, masked) in enumerate([(13, 1e-2, True), (17, 5e-3, False), (19, 2e-2, True)]):
        cfg = small_cfg(3, "CDF44", Bs=16, penal=1 if masked else 0, jmin=2, jmax=3)
        cfg.C_eta = 1e-2
        cfg.nu = nu
        cfg.rhs_precision = 1
        lv, co = grids.random_graded(3, cfg.Jmin, cfg.Jmax, seed=seed, frac=0.3)
        data = smooth_state(cfg, lv, co, 60 + k)
        mask = sphere_mask(cfg, lv, co, [0.5, 0.6, 0.7], 0.25) if masked else None
        solves.append((cfg, lv, co, data, mask))
    cap = sum(len(s[1]) for s in solves) + 8
    assert 4 * (cap - 8) > 4 * 152      # several slabs per SM
    out = []
    for forms in (["tile"] * 4, ["pipe"] * 4, ["direct", "pipe", "tile", "pipe"]):
        with Context(solves[0][0], cap) as ctx:
            ctx.set_stage_forms(forms)
            fs = [_load(ctx, *s) for s in solves]
            ctx.run(fs, 3, use_graph=True)
            out.append([(f.download(), f.time()) for f in fs])
    for res in out[1:]:
        for (u, t), (u0, t0) in zip(res, out[0]):
            assert t == t0
            assert np.array_equal(u, u0)
