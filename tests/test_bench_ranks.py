"""The replica reductions of bench.py under torchrun (N > 1): every rank
times its own replica, the job's time is the maximum over the ranks and its
value the sum; here two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, w = bench.dist_init(world)
    bench.barrier(w)
    out[rank] = (r, w, bench.max_over_ranks(1.5 + rank, w), bench.sum_over_ranks(10.0 * (rank + 1), w))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_sum():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    assert res[0] == (0, 2, 2.5, 30.0)
    assert res[1] == (1, 2, 2.5, 30.0)
