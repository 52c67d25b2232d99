"""Contexts used from several host threads at once (one context per thread,
each on its own stream): a CDF4,0 and a CDF4,4 context run indicators,
refinements and adaptations concurrently, and every result equals the same
sequence run alone. The wavelet filters of a launch are launch parameters,
so no call can see another's taps."""
import threading

import numpy as np
import pytest

from helpers import small_cfg, smooth_state
from wabbit_gb300 import grids
from wabbit_gb300.solver import Context

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def _sequence(w, rounds=3):
    """indicator, refinement and adaptation on one tree, several times"""
    cfg = small_cfg(2, w, Bs=16, jmin=2, jmax=5)
    lv, co = grids.random_graded(2, cfg.Jmin, 4, seed=51, frac=0.3)
    out = []
    with Context(cfg, 8 * len(lv) + 64) as ctx:
        ctx.set_variant(False)
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(smooth_state(cfg, lv, co, 53))
        for r in range(rounds):
            f.sync_ghosts_tree()
            fl, det = f.coarseningIndicator(np.full(cfg.neq, 1e-3))
            out.append((fl, det))
            f.refine_everywhere()
            n = f.adapt(np.full(cfg.neq, 2e-3 * (r + 1)))
            glv, gco = f.grid()
            out.append((glv, gco, f.download()))
    return out


def _same(a, b):
    return len(a) == len(b) and all(
        all(np.array_equal(x, y) for x, y in zip(p, q)) for p, q in zip(a, b))


def test_two_contexts_two_threads_two_wavelets():
    alone = {w: _sequence(w) for w in ("CDF40", "CDF44")}
    res, errs = {}, []

    def run(w):
        try:
            res[w] = _sequence(w)
        except Exception as e:   # reported below
            errs.append(e)

    for _ in range(2):
        th = [threading.Thread(target=run, args=(w,)) for w in ("CDF40", "CDF44", "CDF40")]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
        for w in ("CDF40", "CDF44"):
            assert _same(res[w], alone[w]), w
