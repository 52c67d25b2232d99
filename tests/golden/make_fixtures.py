#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference's own
committed regression files (read-only reference checkout).

Run once in a container that holds the reference checkout:

    python tests/golden/make_fixtures.py /path/to/reference

The fixtures are the reference's HDF5 field files converted to compact numpy
archives, so that the tests (and the GPU machine, which has no reference) can
compare against them:

* vortex2d_equi.npz -- TESTING/acm/3vortices/3vorticesEquiFD4_CDF40: 2-D ACM,
  FD_4th_central, skew-symmetric, Bs=32, 64 blocks on level 3, state at t=10
  (input) and t=20 (output), the (iteration, time) pairs printed in the
  reference's run log (log.original.txt), which pin the time-step sequence,
  and the key/value pairs of its PARAMS_3vortices.ini.
* tg3d_equi.npz -- TESTING/acm/taylorGreen/taylorGreenEqui_FD4_CDF40: 3-D ACM,
  Bs=20, 8 blocks on level 1, state at t=0 (input) and t=10 (output).
* wavelet_adaptive.npz -- TESTING/wavelets: a 2-D adaptive vorticity field
  (112 blocks, levels 2-5, Bs=32), the reference's refine-everywhere results
  with CDF40, CDF20 and CDF60 (448 blocks) and its coarsen-everywhere
  results with CDF20, CDF22, CDF40, CDF42, CDF44, CDF60 and CDF62.
* vortex2d_adapt.npz -- TESTING/acm/3vortices/3vorticesAdaptFD4_CDF40 and
  _CDF42: the adaptive 2-D loop (significant refinement, coarse extension and
  security zone): the ini text and the states at t=10 and t=15.
* acm_cyl.npz -- TESTING/acm/acm_CDF40, acm_CDF44, acm_significant_CDF44
  and acm_norm_CDF44: 2-D ACM flow past a cylinder (convective
  FD_4th_central, penalisation with cosine smoothing, p-norm sponge,
  adaptation every step with mask thresholding and max-level dealiasing,
  Bs=26): the text of acm_cyl.ini, the state at t=0 (input) and the saved
  outputs (t=0.05 and 0.1 for Jmax=6; t=0.2 for the Jmax=5 variants with
  refinement "significant" and with the vector-group norm 2 2 1) with their
  iteration counts, refinement status and saved mask (chi). Each case is
  stored under the prefix "CDF40_" / "CDF44_" / "SIG44_" / "NORM44_".

* h5_files.npz -- every dataset and every attribute of two field files as
  the reference's saveHDF5_tree wrote them (2-D: acm_CDF40/mask_000000000000
  .h5, 3-D: taylorGreen/taylorGreenEqui_FD4_CDF40/ux_000000000000.h5),
  under the prefixes "f2_" / "f3_" ("ds_<name>", "at_<name>"), for the
  writer's tests.

Block data are stored as interiors only, shape (Nb, ncomp, [Bs,] Bs, Bs),
x fastest; block geometry as level (Nb,) and integer coords (Nb, 3).
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from wabbit_gb300.h5io import read_wabbit  # noqa: E402


def _interior(d):
    """Drop the redundant +1 point the writer appends in every direction."""
    b = d["blocks"]
    if d["dim"] == 2:
        return b[:, :-1, :-1]
    return b[:, :-1, :-1, :-1]


def _coords3(d):
    c = np.zeros((len(d["level"]), 3), np.int32)
    c[:, : d["dim"]] = d["coords"]
    return c


def _fields(folder, names, tag):
    ds = [read_wabbit(os.path.join(folder, f"{n}_{tag}.h5")) for n in names]
    for d in ds[1:]:
        assert np.array_equal(d["level"], ds[0]["level"]) and np.array_equal(d["coords"], ds[0]["coords"])
    data = np.stack([_interior(d) for d in ds], axis=1)
    return ds[0], data


def _sorted(d, data):
    """Order blocks by (level, z, y, x) so files with different block orders compare."""
    c = _coords3(d)
    order = np.lexsort((c[:, 0], c[:, 1], c[:, 2], d["level"]))
    return d["level"][order].astype(np.int32), c[order], data[order]


def vortex2d(ref):
    folder = os.path.join(ref, "TESTING/acm/3vortices/3vorticesEquiFD4_CDF40")
    d0, u0 = _fields(folder, ["ux", "uy", "p"], "000010000000")
    d1, u1 = _fields(folder, ["ux", "uy", "p"], "000020000000")
    lv0, c0, u0 = _sorted(d0, u0)
    lv1, c1, u1 = _sorted(d1, u1)
    assert np.array_equal(lv0, lv1) and np.array_equal(c0, c1)
    its, times = [], []
    with open(os.path.join(folder, "log.original.txt"), errors="ignore") as f:
        for line in f:
            m = re.match(r"RUN: it=\s*(\d+) time=\s*([0-9.]+)", line)
            if m:
                its.append(int(m.group(1)))
                times.append(float(m.group(2)))
    from wabbit_gb300.config import _parse_ini
    with open(os.path.join(folder, "PARAMS_3vortices.ini"), errors="ignore") as f:
        kv = _parse_ini(f.read())
    np.savez_compressed(
        os.path.join(HERE, "vortex2d_equi.npz"),
        ini_sec=np.array([k[0] for k in kv]), ini_key=np.array([k[1] for k in kv]),
        ini_val=np.array(list(kv.values())),
        level=lv0, coords=c0, u_in=u0, u_out=u1, t_in=d0["time"], t_out=d1["time"],
        iteration_in=d0["iteration"], iteration_out=d1["iteration"],
        log_it=np.array(its, np.int64), log_time=np.array(times), domain=d0["domain"], Bs=d0["Bs"])


def tg3d(ref):
    folder = os.path.join(ref, "TESTING/acm/taylorGreen/taylorGreenEqui_FD4_CDF40")
    d0, u0 = _fields(folder, ["ux", "uy", "uz", "p"], "000000000000")
    d1, u1 = _fields(folder, ["ux", "uy", "uz", "p"], "000010000000")
    lv0, c0, u0 = _sorted(d0, u0)
    lv1, c1, u1 = _sorted(d1, u1)
    assert np.array_equal(lv0, lv1) and np.array_equal(c0, c1)
    np.savez_compressed(
        os.path.join(HERE, "tg3d_equi.npz"),
        level=lv0, coords=c0, u_in=u0, u_out=u1, t_in=d0["time"], t_out=d1["time"],
        iteration_out=d1["iteration"], domain=d0["domain"], Bs=d0["Bs"])


def wavelets(ref):
    folder = os.path.join(ref, "TESTING/wavelets")
    out = {}
    d = read_wabbit(os.path.join(folder, "vor_000020000000.h5"))
    lv, c, u = _sorted(d, _interior(d)[:, None])
    out.update(in_level=lv, in_coords=c, in_u=u, domain=d["domain"], Bs=d["Bs"])
    d = read_wabbit(os.path.join(folder, "adaptive_CDF40", "vor_00100.h5"))
    lv, c, u = _sorted(d, _interior(d)[:, None])
    out.update(refined_level=lv, refined_coords=c, refined_u=u)
    for w in ["CDF20", "CDF60"]:   # the refinement with the order-2 and order-6 predictors
        d = read_wabbit(os.path.join(folder, f"adaptive_{w}", "vor_00100.h5"))
        lv, c, u = _sorted(d, _interior(d)[:, None])
        out.update({f"refined_{w}_level": lv, f"refined_{w}_coords": c, f"refined_{w}_u": u})
    for w in ["CDF20", "CDF22", "CDF40", "CDF42", "CDF44", "CDF60", "CDF62"]:
        d = read_wabbit(os.path.join(folder, f"adaptive_{w}", "vor_00200.h5"))
        lv, c, u = _sorted(d, _interior(d)[:, None])
        out.update({f"coarsened_{w}_level": lv, f"coarsened_{w}_coords": c, f"coarsened_{w}_u": u})
    np.savez_compressed(os.path.join(HERE, "wavelet_adaptive.npz"), **out)


def _status(folder, tag, d):
    """The refinement_status dataset of a field file, in the order _sorted
    gives its blocks."""
    from wabbit_gb300.h5io import H5File
    st = H5File(os.path.join(folder, f"ux_{tag}.h5")).read("refinement_status").astype(np.int32)
    c = _coords3(d)
    return st[np.lexsort((c[:, 0], c[:, 1], c[:, 2], d["level"]))]


def acm_cyl(ref):
    out = {}
    cases = [("CDF40", "acm_CDF40", [("000000000000", "t0"), ("000000050000", "t1"), ("000000100000", "t2")]),
             ("CDF44", "acm_CDF44", [("000000000000", "t0"), ("000000050000", "t1"), ("000000100000", "t2")]),
             ("SIG44", "acm_significant_CDF44", [("000000000000", "t0"), ("000000200000", "t2")]),
             ("NORM44", "acm_norm_CDF44", [("000000000000", "t0"), ("000000200000", "t2")])]
    for w, sub, tags in cases:
        folder = os.path.join(ref, "TESTING/acm", sub)
        with open(os.path.join(folder, "acm_cyl.ini"), errors="ignore") as f:
            out[f"{w}_ini"] = np.array(f.read())
        for tag, key in tags:
            d, u = _fields(folder, ["ux", "uy", "p"], tag)
            st = _status(folder, tag, d)
            lv, c, u = _sorted(d, u)
            dm = read_wabbit(os.path.join(folder, f"mask_{tag}.h5"))
            lvm, cm, m = _sorted(dm, _interior(dm)[:, None])
            assert np.array_equal(lv, lvm) and np.array_equal(c, cm)
            out.update({f"{w}_{key}_level": lv, f"{w}_{key}_coords": c, f"{w}_{key}_u": u,
                        f"{w}_{key}_chi": m[:, 0], f"{w}_{key}_time": d["time"],
                        f"{w}_{key}_iteration": d["iteration"], f"{w}_{key}_status": st})
    np.savez_compressed(os.path.join(HERE, "acm_cyl.npz"), **out)


def vortex2d_adapt(ref):
    """TESTING/acm/3vortices/3vorticesAdaptFD4_CDF40 (and _CDF42): the
    adaptive 2-D loop (significant refinement, coarse extension and security
    zone) from t=10 to t=15: the ini text and both saved states; the CDF4,2
    case's entries carry the prefix CDF42_."""
    out = {}
    for w, pre in [("CDF40", ""), ("CDF42", "CDF42_")]:
        folder = os.path.join(ref, f"TESTING/acm/3vortices/3vorticesAdaptFD4_{w}")
        with open(os.path.join(folder, "PARAMS_3vortices.ini"), errors="ignore") as f:
            out[pre + "ini"] = np.array(f.read())
        for tag, key in [("000010000000", "t10"), ("000015000000", "t15")]:
            d, u = _fields(folder, ["ux", "uy", "p"], tag)
            lv, c, u = _sorted(d, u)
            out.update({f"{pre}{key}_level": lv, f"{pre}{key}_coords": c, f"{pre}{key}_u": u,
                        f"{pre}{key}_time": d["time"], f"{pre}{key}_iteration": d["iteration"]})
    np.savez_compressed(os.path.join(HERE, "vortex2d_adapt.npz"), **out)


def h5_files(ref):
    from wabbit_gb300.h5io import H5File
    out = {}
    for tag, rel in [("f2", "TESTING/acm/acm_CDF40/mask_000000000000.h5"),
                     ("f3", "TESTING/acm/taylorGreen/taylorGreenEqui_FD4_CDF40/ux_000000000000.h5")]:
        h = H5File(os.path.join(ref, rel))
        for name in h.datasets:
            out[f"{tag}_ds_{name}"] = h.read(name)
            for a, v in h.attrs(name).items():
                out[f"{tag}_at_{a}"] = np.atleast_1d(v)
    np.savez_compressed(os.path.join(HERE, "h5_files.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <path of the reference checkout>")
    ref = sys.argv[1]
    vortex2d(ref)
    tg3d(ref)
    wavelets(ref)
    acm_cyl(ref)
    vortex2d_adapt(ref)
    h5_files(ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
