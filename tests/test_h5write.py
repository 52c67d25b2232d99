"""The HDF5 writer (saveHDF5_tree's file layout, LIB/MESH/InputOutput.f90:
1-309, chunked as module_hdf5_wrapper.f90:261-293): files it writes read back
bit for bit, and re-writing the content of two of the reference's own field
files reproduces every dataset and attribute of the originals."""
import os

import numpy as np
import pytest

from wabbit_gb300 import grids, h5io


def test_write_read_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    ds = {"a": rng.standard_normal((300, 17, 17)), "b": np.arange(300, dtype=np.int32),
          "c": (np.arange(300, dtype=np.int64) << 33) - 5, "d": rng.standard_normal((3, 2))}
    at = {"a": {"time": np.array([1.5]), "dim": np.array([2], np.int32), "v": np.arange(3, dtype=np.int32)}}
    p = str(tmp_path / "x.h5")
    h5io.write_h5(p, ds, at)
    h = h5io.H5File(p)
    assert sorted(h.datasets) == sorted(ds)
    for k, v in ds.items():
        r = h.read(k)
        assert r.dtype == v.dtype and np.array_equal(r, v)
        assert h.datasets[k].chunk[:-1] == tuple(min(n, 128) for n in v.shape)
    for k, v in at["a"].items():
        assert np.array_equal(np.atleast_1d(h.attrs("a")[k]), v)


def test_many_chunks_two_level_btree(tmp_path):
    """More chunks than one B-tree node holds (64): an internal level."""
    big = np.random.default_rng(1).standard_normal((9000, 5, 5))
    p = str(tmp_path / "big.h5")
    h5io.write_h5(p, {"blocks": big})
    assert np.array_equal(h5io.H5File(p).read("blocks"), big)


@pytest.mark.parametrize("dim", [2, 3])
def test_save_wabbit_round_trip(tmp_path, dim):
    lv, co = grids.random_graded(dim, 2, 4 if dim == 2 else 3, seed=5, frac=0.4)
    Bs = [12, 10, 8][:dim]
    dom = [1.0, 2.0, 3.0][:dim]
    rng = np.random.default_rng(2)
    blocks = rng.standard_normal((len(lv),) + tuple(b + 1 for b in Bs[::-1]))
    p = str(tmp_path / f"ux_{h5io.timestr(0.25)}.h5")
    assert p.endswith("ux_000000250000.h5")
    h5io.save_wabbit(p, blocks, lv, co, 0.25, 17, dom, Bs, max_level=4)
    d = h5io.read_wabbit(p)
    assert np.array_equal(d["blocks"], blocks)
    assert np.array_equal(d["level"], lv) and np.array_equal(d["coords"], np.asarray(co)[:, :dim])
    assert d["time"] == 0.25 and d["iteration"] == 17 and d["dim"] == dim and d["max_level"] == 4
    assert np.array_equal(d["domain"], dom) and np.array_equal(d["Bs"], Bs)


@pytest.mark.parametrize("tag", ["f2", "f3"])
def test_rewrite_reference_files(golden, tmp_path, tag):
    """Every dataset and attribute of the reference's file (as the reader
    reads it) from save_wabbit given only the blocks, the grid, the time
    stamp and the per-block bookkeeping the file carries."""
    z = golden("h5_files.npz")
    ds = {k[len(tag) + 4:]: z[k] for k in z.files if k.startswith(f"{tag}_ds_")}
    at = {k[len(tag) + 4:]: z[k] for k in z.files if k.startswith(f"{tag}_at_")}
    dim = int(at["dim"][0])
    Bs = at["block-size"][:dim]
    dom = at["domain-size"]
    # level and integer coordinates from the file's own origin and spacing
    spacing = ds["coords_spacing"][:, ::-1]
    origin = ds["coords_origin"][:, ::-1]
    level = ds["level"].astype(np.int64)
    coords = np.rint(origin / (spacing * Bs)).astype(np.int64)
    p = str(tmp_path / "re.h5")
    h5io.save_wabbit(p, ds["blocks"], level, coords, float(at["time"][0]), int(at["iteration"][0]), dom, Bs,
                     int(at["max_level"][0]), refinement_status=ds["refinement_status"], lgt_ids=ds["lgt_ids"],
                     procs=ds["procs"])
    h = h5io.H5File(p)
    assert sorted(h.datasets) == sorted(ds)
    for k, v in ds.items():
        r = h.read(k)
        assert r.dtype == v.dtype and r.shape == v.shape, k
        assert np.array_equal(r, v), k
    a = h.attrs("blocks")
    assert sorted(a) == sorted(at)
    for k, v in at.items():
        got = np.atleast_1d(a[k])
        assert got.dtype == v.dtype and np.array_equal(got, v), k
    # and the reader's view of both files agrees
    ref = str(tmp_path / "orig.h5")
    h5io.write_h5(ref, ds, {"blocks": at})
    a1, a2 = h5io.read_wabbit(ref), h5io.read_wabbit(p)
    for k in ("blocks", "level", "coords", "origin", "spacing", "domain", "Bs"):
        assert np.array_equal(a1[k], a2[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_checkpoint_restart_on_device(tmp_path, dim):
    """save_hdf5 from a context, load_hdf5 into a fresh one: same grid,
    interior state and time bit for bit, and the restarted run continues
    exactly as the original."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from helpers import small_cfg, smooth_state
    from wabbit_gb300.solver import Context
    cfg = small_cfg(dim, "CDF40", Bs=8, jmin=1, jmax=3)
    lv, co = grids.random_graded(dim, 1, 3, seed=8, frac=0.4)
    data = smooth_state(cfg, lv, co, 9)
    with Context(cfg, 4 * len(lv)) as ctx:
        f = ctx.forest()
        f.set_grid(lv, co)
        f.upload(data)
        f.set_time(0.0)
        f.run(2, use_graph=False)
        paths = f.save_hdf5(str(tmp_path), iteration=2)
        assert len(paths) == cfg.neq and all(os.path.exists(p) for p in paths)
        u_saved = f.download_interior()
        t_saved = f.time()[0]
        f.run(2, use_graph=False)
        u_cont = f.download_interior()
        g = ctx.forest()
        it = g.load_hdf5(paths)
        assert it == 2 and g.time()[0] == t_saved
        assert np.array_equal(g.grid()[0], f.grid()[0]) and np.array_equal(g.grid()[1], f.grid()[1])
        assert np.array_equal(g.download_interior(), u_saved)
        g.run(2, use_graph=False)
        assert np.array_equal(g.download_interior(), u_cont)
