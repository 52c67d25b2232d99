"""Serving loop: solves admitted by HBM footprint as they arrive, stepped in
batched launches beside each other. Each served result must be identical to
the same solve run alone (same step chunks), and the arena limit must make
later requests wait for earlier ones to finish."""
import numpy as np
import pytest

from wabbit_gb300 import serving
from wabbit_gb300.serving import Request

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


def test_served_equals_alone_and_admission_waits():
    reqs = [
        Request(0, 0.00, 3, 0, 101, 1e-3, nsteps=10),
        Request(1, 0.00, 2, 1, 102, 2e-3, nsteps=10),
        Request(2, 0.01, 3, 0, 103, 4e-3, nsteps=10),
        Request(3, 0.02, 3, 1, 104, 7e-4, nsteps=10),   # 960 blocks: waits for a 512-block solve
        Request(4, 0.02, 2, 0, 105, 5e-3, nsteps=15),
    ]
    srv = serving.Server(budget_gb=2.3, chunk=5, keep_results=True, workers={3: 1, 2: 1})
    try:
        assert 1024 <= srv.capacity[3] < 1472
        recs, summ = srv.run(reqs, realtime=False)
    finally:
        srv.close()
    assert summ["requests"] == len(reqs)
    # request 3 only fits after one of the first two 3-D solves has left
    assert recs[3]["admitted"] >= min(recs[0]["done"], recs[2]["done"])
    for r in reqs:
        u, t = serving.solve_alone(r, chunk=5)
        assert np.array_equal(recs[r.rid]["u"], u), r.rid
        assert recs[r.rid]["time"] == t
        assert np.isfinite(u).all() and np.abs(u).max() > 0


def test_stream_is_seeded():
    a = serving.make_stream(16, seed=4)
    b = serving.make_stream(16, seed=4)
    assert [(r.arrival, r.dim, r.size, r.seed, r.nu) for r in a] == [(r.arrival, r.dim, r.size, r.seed, r.nu) for r in b]
    assert all(5e-4 <= r.nu <= 5e-3 for r in a)
    assert np.all(np.diff([r.arrival for r in a]) > 0)


def test_served_with_adaptation_equals_alone():
    """With the reference's adaptation cycle every 5 steps (sync, refine
    everywhere, 5 RK4 steps, adapt_tree; the 3-D solve with the lifted
    CDF4,4 algorithm) a served solve still equals the same solve alone: grid
    and state."""
    reqs = [
        Request(0, 0.00, 3, 1, 201, 1e-3, nsteps=10),
        Request(1, 0.00, 2, 1, 202, 2e-3, nsteps=10),
        Request(2, 0.01, 2, 3, 203, 3e-3, nsteps=15),
    ]
    srv = serving.Server(budget_gb=16.0, keep_results=True, adapt_every=5)
    try:
        recs, summ = srv.run(reqs, realtime=False)
    finally:
        srv.close()
    assert summ["requests"] == len(reqs)
    for r in reqs:
        u, t = serving.solve_alone(r, adapt_every=5)
        assert recs[r.rid]["u"].shape == u.shape, r.rid
        assert np.array_equal(recs[r.rid]["u"], u), r.rid
        assert recs[r.rid]["time"] == t
        assert np.isfinite(u).all() and np.abs(u).max() > 0


def test_several_contexts_per_geometry_equal_alone():
    """Two 3-D contexts (the first sized for the largest request, each served
    by its own host thread) with the adaptation cycle: every served solve
    equals the same solve alone, and both contexts take requests."""
    reqs = [Request(i, 0.005 * i, 3, i % 2, 300 + i, 1e-3 * (1 + i), nsteps=10) for i in range(6)]
    reqs.append(Request(6, 0.0, 2, 1, 306, 2e-3, nsteps=10))
    srv = serving.Server(budget_gb=24.0, keep_results=True, adapt_every=5, workers={3: 2, 2: 1})
    try:
        assert len(srv.workers[3]) == 2
        recs, summ = srv.run(reqs, realtime=False)
    finally:
        srv.close()
    assert summ["requests"] == len(reqs)
    assert {recs[r.rid]["worker"] for r in reqs if r.dim == 3} == {0, 1}
    for r in reqs:
        u, t = serving.solve_alone(r, adapt_every=5)
        assert np.array_equal(recs[r.rid]["u"], u), r.rid
        assert recs[r.rid]["time"] == t
