#!/usr/bin/env python3
"""Benchmark of the ACM block-level time stepper (point-updates/s).

A step is one RK4 time step (timeStep_tree: ghost sync, dt, four RHS+RK
stages) over every block of the workload grid. The default workload is the
batched mixed-precision configuration: the 3-D ACM channel with a penalised
sphere (Bs=16^3, g=6, CDF4,4) at Jmax=7, 36,688 blocks over five levels, the
stencils and stage arithmetic in double-float on the FP32 units with the
FP64 state, the RK4 step captured as one CUDA graph (see
wabbit_gb300/workloads.py). `--workload acm3d_sphere` runs the FP64
configuration at Jmax=6 (4,208 blocks).

value: point-updates/s with the state resident in HBM, K steps replayed from
       a captured CUDA graph, timed with CUDA events on the solver's stream.
e2e:   the same through the C ABI with host buffers: wg_rk4_stream over a
       stream of at least 40 steps, every step's input copied in from pinned
       host memory and its result copied out to pinned host memory (the
       copies of neighbouring steps overlap the step on the device);
       e2e.sequential: wg_upload_interior + wg_rk4_step +
       wg_download_interior one after another.
plain_fp64: the plain per-solve FP64 path on the same grid and IC (one
       wg_rk4_step call per step, no graph), its speed and the relative L2
       difference of the two states after K steps.
roofline: the RK-stage kernels against the measured HBM copy bandwidth:
       algorithmic bytes of one stage (5 state vectors, the ghost halo and the
       mask of masked blocks per point) over the mean device time of the four
       stages' kernels in profiled steps (CUDA events between the kernel
       groups). traffic: DRAM bytes of the stage kernels measured in the run
       by a one-pass ncu capture of the same workload at Jmax=5, scaled to the
       full grid by points. For the FP64 precision also the FP64 rate against
       the FP64 FMA peak measured in the same run.
cpu_baseline: the CPU oracle (a scalar C++ restatement of the reference's
       Fortran, OpenMP over blocks) on a bounded sample of the same physics.

--impl reference runs only the CPU oracle (the reference is Fortran and
cannot be built here; the oracle reproduces its regression outputs bit for
bit) on the same metric.
"""
import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic cost of one RK stage per interior point (FP64, fused ideal):
# read stage input, u_n and the accumulator, write accumulator and next stage
# input: 5 state vectors of neq doubles; masked blocks also read 6 mask words
WORDS_PER_POINT_STAGE = 5
MASK_WORDS = 6
# FP64 operations of the FD_4th_central RHS + RK update per point and stage
FLOPS_PER_POINT_STAGE = {2: 118, 3: 238}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="acm3d_sphere_j7")
    ap.add_argument("--variant", choices=["fast", "strict"], default="fast")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--jmax", type=int, default=None, help="override the workload's Jmax (smaller cases)")
    ap.add_argument("--precision", choices=["fp64", "fp32"], default=None,
                    help="RHS stencil precision (default: the workload's; fp32 = double-float on the FP32 units)")
    ap.add_argument("--rate", type=float, default=8.0, help="serving: Poisson arrival rate (requests/s)")
    ap.add_argument("--requests", type=int, default=256, help="serving: number of requests")
    ap.add_argument("--budget-gb", type=float, default=160.0, help="serving: HBM budget of the arenas")
    ap.add_argument("--serving-requests", type=int, default=24,
                    help="default workload: requests of the short serving stream run after it (0: none)")
    ap.add_argument("--adapt-every", type=int, default=5,
                    help="serving: adaptation cycle length in steps (0: no adaptation)")
    ap.add_argument("--stage-form", default="auto",
                    help="FP32-pipe stage kernel form: auto (timed per RK stage), direct, tile, march, pipe, tile2, "
                         "tile8, or four "
                         "comma-separated forms for RK stages 1-4")
    ap.add_argument("--traffic", choices=["auto", "off"], default="auto",
                    help="measure the stage kernels' DRAM bytes with a one-pass ncu capture (dram__bytes_read/"
                         "write) of one RK4 step of the workload at Jmax=5, scaled to the full grid by points")
    ap.add_argument("--traffic-case", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--compare-plain", choices=["auto", "on", "off"], default="auto",
                    help="also time the plain per-solve FP64 path (one wg_rk4_step call per step, no graph) "
                         "and report the speed-up and the L2 difference of the two after K steps "
                         "(auto: on for the FP32-pipe precision)")
    return ap.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons (200 ms)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        try:
            with open(self.out.name) as f:
                rows = [r.strip().split(",") for r in f if r.strip()]
        except OSError:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def set_forms(ctx, spec):
    """Apply a --stage-form value to a context."""
    if "," in spec:
        ctx.set_stage_forms(spec.split(","))
    else:
        ctx.set_stage_form(spec)


TRAFFIC_JMAX = 5


def run_traffic_case(args):
    """The small case the traffic capture profiles: the workload at Jmax=5,
    the given stage forms, one RK4 step of batched launches without a graph
    (two launches per RK stage, unmasked and masked blocks; one in the pipe
    form). Prints the
    grid's sizes as JSON."""
    import torch
    from wabbit_gb300 import build, workloads
    from wabbit_gb300.solver import Context
    build.build()
    torch.cuda.set_device(0)
    cfg, lv, co, u0, ids, masks = workloads.build(args.workload, jmax=TRAFFIC_JMAX)
    ctx = Context(cfg, len(lv) + 16)
    set_forms(ctx, args.stage_form)
    f = ctx.forest()
    f.set_grid(lv, co)
    f.upload_interior(u0)
    if masks is not None and len(ids):
        f.set_mask_sparse(ids, masks)
    f.set_time(0.0)
    f.run(1, use_graph=False)
    ctx.synchronize()
    npts = len(lv) * int(np.prod([cfg.Bs[d] for d in range(cfg.dim)]))
    print(json.dumps({"blocks": len(lv), "points": npts, "masked_blocks": f.stats()[1]}))
    ctx.close()


def measure_traffic(args, forms):
    """DRAM bytes of each RK stage's kernels per interior point, from ncu on
    the small case (one pass: two DRAM counters of one unit, the 8 stage
    launches of one step -- unmasked and masked blocks per stage -- no replay
    of device memory). The small case is first run without ncu and must exit
    0. Returns (per-stage bytes per point, description) or (None, reason)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--traffic-case", "--workload", args.workload,
           "--stage-form", ",".join(forms)]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    except subprocess.TimeoutExpired:
        return None, "the small case did not finish without ncu"
    if r.returncode != 0:
        return None, "the small case failed without ncu: " + r.stderr.strip()[-200:]
    info = json.loads(r.stdout.strip().splitlines()[-1])
    ncu = shutil.which("ncu") or "/usr/local/cuda/bin/ncu"
    if not os.path.exists(ncu):
        return None, "ncu not found"
    log = tempfile.NamedTemporaryFile(prefix="traffic", suffix=".csv", delete=False).name
    # launches per RK stage: unmasked and masked blocks, or one (pipe form)
    per = [1 if fm == "pipe" else 2 for fm in forms]   # launches per RK stage
    ncmd = [ncu, "--metrics", "dram__bytes_read.sum,dram__bytes_write.sum", "--clock-control", "none",
            "-k", "regex:acm_stage_df", "-c", str(sum(per)), "--csv", "--print-units", "base", "--log-file", log] + cmd
    try:
        r = subprocess.run(ncmd, capture_output=True, text=True, timeout=900)
    except subprocess.TimeoutExpired:
        return None, "ncu capture did not finish"
    if r.returncode != 0:
        return None, "ncu failed: " + (r.stderr.strip() or r.stdout.strip())[-200:]
    import csv
    launches = {}
    with open(log) as fh:
        rows = [row for row in csv.reader(fh)]
    hdr = None
    for row in rows:
        if row and row[0] == "ID":
            hdr = row
            continue
        if hdr is None or len(row) != len(hdr):
            continue
        d = dict(zip(hdr, row))
        if d.get("Metric Name") in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
            launches.setdefault(int(d["ID"]), 0.0)
            launches[int(d["ID"])] += float(d["Metric Value"].replace(",", ""))
    os.unlink(log)
    ids = sorted(launches)
    if len(ids) != sum(per):
        return None, f"expected {sum(per)} stage launches in the capture, got {len(ids)}"
    per_stage, at = [], 0
    for j in range(4):
        per_stage.append(sum(launches[ids[at + k]] for k in range(per[j])) / info["points"])
        at += per[j]
    desc = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the {sum(per)} stage launches (RK stages 1-4; "
            f"unmasked and masked blocks apart except in the pipe form) of one step of {args.workload} at "
            f"Jmax={TRAFFIC_JMAX} ({info['blocks']} blocks, {info['masked_blocks']} masked), per interior point, "
            f"scaled to the full grid by its points")
    return per_stage, desc


# --------------------------------------------------------------------- CPU
def oracle_for(workload, jmax=None, threads=None):
    """The oracle (the reference's algorithm restated in C++, OpenMP over
    blocks in the ghost sync, RHS, RK update and dt) loaded with the
    workload's grid, initial condition and sparse mask. Returns (oracle,
    interior points)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from wabbit_gb300 import workloads
    cfg, lv, co, u, ids, masks = workloads.build(workload, jmax=jmax)
    threads = threads or os.cpu_count() or 1
    o = pyoracle.Oracle(cfg, threads=threads)
    o.set_grid(lv, co, None)
    o.set_interior(u)
    del u
    if masks is not None and len(ids):
        o.set_mask_sparse(ids, masks)
    npts = len(lv) * int(np.prod([cfg.Bs[d] for d in range(cfg.dim)]))
    return o, npts, cfg, len(lv)


def oracle_bytes(workload, jmax):
    """Host bytes the oracle needs for the workload at jmax (state with g
    ghost layers, five interior RK registers, the initial condition)."""
    from wabbit_gb300 import workloads
    cfg = workloads.make_config(workload)
    cfg.Jmax = jmax
    lv, _ = workloads.make_grid(workload, cfg)
    dim = cfg.dim
    full = int(np.prod([cfg.Bs[d] + 2 * cfg.g for d in range(dim)]))
    inner = int(np.prod([cfg.Bs[d] for d in range(dim)]))
    return 8.0 * len(lv) * cfg.neq * (full + 5 * inner + 2 * inner) * 1.15


def host_mem_available():
    """Bytes this process may still allocate: MemAvailable, capped by a
    cgroup memory limit if one is set."""
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = float(line.split()[1]) * 1024
    except OSError:
        pass
    try:
        with open("/sys/fs/cgroup/memory.max") as f:
            lim = f.read().strip()
        with open("/sys/fs/cgroup/memory.current") as f:
            cur = float(f.read().strip())
        if lim != "max":
            room = float(lim) - cur
            avail = room if avail is None else min(avail, room)
    except OSError:
        pass
    return avail


def time_oracle(o, steps, warmup=1, seconds=None):
    """Warm-up steps, then `steps` RK4 steps (or as many as fit in
    `seconds`, at least one); returns (steps, wall seconds)."""
    t = 0.0
    for _ in range(warmup):
        t, _ = o.step(t)
    n = 0
    t0 = time.perf_counter()
    while True:
        t, _ = o.step(t)
        n += 1
        el = time.perf_counter() - t0
        if (seconds is None and n >= steps) or (seconds is not None and (el >= seconds or n >= steps)):
            return n, el


def cpu_sample(workload, seconds=12.0, threads=None):
    """Time the oracle on a bounded sample: the workload's physics on its
    Jmax=5 grid (same block size, ghost width, IC and mask), RK4 steps on
    all host cores until `seconds` of wall time have been spent; and the
    one-core rate on the Jmax=4 grid."""
    threads = threads or os.cpu_count() or 1
    o, npts, cfg, nblk = oracle_for(workload, jmax=5, threads=threads)
    steps, el = time_oracle(o, 200, 1, seconds)
    value = npts * steps / el
    del o
    o1, npts1, _, nblk1 = oracle_for(workload, jmax=4, threads=1)
    steps1, el1 = time_oracle(o1, 50, 1, seconds / 2)
    sample = (f"{workload} physics (IC, mask, block size, ghosts) on its Jmax=5 grid ({nblk} blocks, {npts} "
              f"points), {steps} RK4 steps in {el:.1f} s on {threads} threads; one core: Jmax=4 grid "
              f"({nblk1} blocks), {steps1} steps in {el1:.1f} s")
    return value, threads, sample, el / steps, npts1 * steps1 / el1


# --------------------------------------------------------------------- GPU
def run_ours(args, rank, world):
    import torch
    from wabbit_gb300 import build, workloads
    from wabbit_gb300.solver import Context, probe_alu

    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cfg, lv, co, u0, ids, masks = workloads.build(args.workload, jmax=args.jmax)
    if args.precision is not None:
        cfg.rhs_precision = 1 if args.precision == "fp32" else 0
    nblk = len(lv)
    dim = cfg.dim
    npts_blk = int(np.prod([cfg.Bs[d] for d in range(dim)]))
    npts = nblk * npts_blk
    ctx = Context(cfg, nblk + 16)
    ctx.set_variant(args.variant == "fast")
    if cfg.rhs_precision:
        set_forms(ctx, args.stage_form)
    f = ctx.forest()
    f.set_grid(lv, co)
    f.upload_interior(u0)
    if masks is not None and len(ids):
        f.set_mask_sparse(ids, masks)
    _, nmasked = f.stats()
    f.set_time(0.0)
    f.sync_ghosts_RHS_tree()
    stream = torch.cuda.ExternalStream(ctx.stream)

    # warm-up (also captures the graph)
    f.run(max(args.warmup, 1), use_graph=True)
    ctx.synchronize()
    graph_kernels = capi_graph_kernels(ctx)

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    ctx.synchronize()
    with Clocks(local) as clk:
        e0.record(stream)
        f.run(args.steps, use_graph=True)
        e1.record(stream)
        e1.synchronize()
        ctx.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world)
    t_end, dt_last = f.time()  # raises if the run diverged
    value = sum_over_ranks(npts * args.steps / (ms * 1e-3), world)

    # per-kernel-group device times of real steps (events between the
    # groups, same launches as the graph), after the timed region
    nprof = max(3, min(args.steps, 5))
    prof = ctx.step_profile([f], nprof)
    stage_ms = [prof[f"stage{j}"] for j in range(1, 5)]
    mean_stage_ms = float(np.mean(stage_ms))
    # algorithmic bytes of one stage launch (FP64 basis, fused ideal): 5 state
    # vectors of neq words per interior point (stage input, u_n, accumulator
    # read + write, next input), the ghost halo of the stage input read and
    # its sync written ((Bs+2 g_rhs)^d - Bs^d per Bs^d, x 2 x neq words), and
    # 5 mask words per point of the masked blocks
    halo_w = (float(np.prod([cfg.Bs[d] + 2 * cfg.g_rhs for d in range(dim)])) - npts_blk) / npts_blk * 2 * cfg.neq
    mask_bytes = 8.0 * nmasked * npts_blk * 5
    bytes_interior = 8.0 * npts * cfg.neq * WORDS_PER_POINT_STAGE + mask_bytes
    bytes_stage = bytes_interior + 8.0 * npts * halo_w
    flops_stage = float(FLOPS_PER_POINT_STAGE[dim]) * npts
    hbm_peak, hbm_src = measured_peaks()
    ach_gbs = bytes_stage / (mean_stage_ms * 1e-3) / 1e9
    ach_tf = flops_stage / (mean_stage_ms * 1e-3) / 1e12
    form = ctx.stage_forms() if cfg.rhs_precision else ["direct"] * 4
    kname = {"direct": "acm_stage_df_kernel", "tile": "acm_stage_df_tile (TMA slabs)",
             "march": "acm_stage_df_march (TMA plane ring)",
             "pipe": "acm_stage_df_pipe (persistent TMA slab pipeline)",
             "tile2": "acm_stage_df_tile<2> (TMA slabs of 2 planes)", "tile8": "acm_stage_df_tile<8> (TMA slabs of 8 planes)"}
    stage_kernel = ("acm_stage_kernel (FP64)" if cfg.rhs_precision == 0 else
                    ", ".join(kname[x] for x in dict.fromkeys(form)))
    traffic, traffic_src = None, "not measured (--traffic off)"
    if args.traffic == "auto" and cfg.rhs_precision and rank == 0 and world == 1:
        per_pt, traffic_src = measure_traffic(args, form)
        if per_pt is not None:
            traffic = {"per_stage": [v * npts for v in per_pt], "mean": float(np.mean(per_pt)) * npts}

    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
        host_out = [torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
        host_in[...] = u0
        # a stream of at least 40 steps (a host driver streams its whole
        # run): its fill (the first input in) and drain (the last result
        # out) are in the timed region once
        k = max(40, args.steps)
        f.rk4_stream([host_in] * 2, host_out)
        barrier(world)
        t0 = time.perf_counter()
        # every step: its input from pinned host memory, one RK4 step, its
        # result back to pinned host memory (the copies of neighbouring steps
        # overlap the step on the device)
        f.rk4_stream([host_in] * k, [host_out[i % 2] for i in range(k)])
        el = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": sum_over_ranks(npts * k / el, world), "unit": "point-updates/s",
               "h2d_bytes_per_step": int(host_in.nbytes), "d2h_bytes_per_step": int(host_out[0].nbytes),
               "steps": k, "path": "wg_rk4_stream (pinned host buffers; input of step k+1 and result of step k "
                                    "copied while the device steps)"}
        # the same without overlap: upload, step, download one after another
        k2 = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(k2):
            f.upload_interior(host_in)
            f.timeStep_tree()
            f.download_interior(host_out[0])
        el2 = max_over_ranks(time.perf_counter() - t0, world)
        e2e["sequential"] = {"value": sum_over_ranks(npts * k2 / el2, world), "steps": k2,
                             "path": "wg_upload_interior + wg_rk4_step + wg_download_interior"}

    plain = None
    if args.compare_plain == "on" or (args.compare_plain == "auto" and cfg.rhs_precision == 1):
        plain = compare_plain(args, cfg, lv, co, u0, ids, masks, f, ctx, value / max(world, 1), npts)

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        v, cores, sample, _, v1 = cpu_sample(args.workload)
        cpu = {"value": v, "unit": "point-updates/s", "cores": cores, "kind": "port", "sample": sample,
               "one_core_value": v1}

    clocks = clk.summary()
    # bytes one RK stage touches (input, u_n copy, increment, next input)
    state_gb = nblk * cfg.neq * 8.0 * ((cfg.Bs[0] + 2 * cfg.g_rhs) ** dim + 3 * npts_blk) / 1e9
    line = {
        "metric": "ACM point-updates/s/GPU",
        "value": value,
        "unit": "point-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if cfg.rhs_precision == 0 else "f64 state, double-float (2xf32) stencils",
        "data": "synthetic (seeded IC and grid, see wabbit_gb300/workloads.py)",
        "config": {
            "workload": args.workload, "dim": dim, "Bs": list(cfg.Bs)[:dim], "g": cfg.g, "g_rhs": cfg.g_rhs,
            "wavelet": cfg.wavelet.decode(), "Jmax": cfg.Jmax, "blocks": nblk, "points": npts,
            "masked_blocks": nmasked, "levels": np.bincount(lv).tolist(), "variant": args.variant,
            "rhs_precision": "fp64" if cfg.rhs_precision == 0 else "fp32-pipe double-float",
            "stage_forms": form,
            "rk": "RK4", "graph": True,
            "l2": (f"stage buffers {state_gb:.1f} GB > 129 MB L2 (no flush needed)" if state_gb > 0.5 else
                   f"stage buffers {state_gb:.2f} GB: each stage streams more than L2 holds"),
            "parallelism": "replicas" if world > 1 else "1 GPU",
        },
        "roofline": {"bound": "hbm", "achieved": ach_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach_gbs / hbm_peak, "traffic": traffic["mean"] if traffic else None,
                     "kernel": stage_kernel, "stage_forms": form,
                     "launch_ms": mean_stage_ms, "launch_ms_per_stage": stage_ms, "peak_source": hbm_src,
                     "algorithmic_bytes_per_launch": bytes_stage,
                     "bytes_per_point": (f"{WORDS_PER_POINT_STAGE} state words x neq (stage input, u_n, accumulator "
                                         f"read + write, next input) + {halo_w:.2f} halo words (ghost layers read "
                                         f"and written) per interior point, + 5 mask words per point of masked "
                                         f"blocks; x 8 B"),
                     "frac_interior_only": bytes_interior / (mean_stage_ms * 1e-3) / 1e9 / hbm_peak,
                     "frac_per_stage": [bytes_stage / (t * 1e-3) / 1e9 / hbm_peak for t in stage_ms],
                     "timing": f"mean of the 4 stage kernels over {nprof} profiled steps (CUDA events between "
                               f"the kernel groups on the solver stream, after the timed region)",
                     "traffic_per_stage": traffic["per_stage"] if traffic else None,
                     "traffic_source": traffic_src},
        "kernels_ms": prof,
        "gpu_launches": graph_kernels * args.steps,
        "clocks": clocks,
        "t_end": t_end,
        "dt_last": dt_last,
    }
    if cfg.rhs_precision == 0:
        fp64_peak, fp32_peak = probe_alu()
        line["roofline_alu"] = {"bound": "fp64", "achieved": ach_tf, "peak": fp64_peak, "unit": "TFLOP/s",
                                "frac": ach_tf / fp64_peak, "flops_per_launch": flops_stage,
                                "peak_source": "FP64 FMA probe measured in this run (wg_probe_alu)",
                                "fp32_peak_tflops": fp32_peak}
    if e2e is not None:
        line["e2e"] = e2e
    if plain is not None:
        line["plain_fp64"] = plain
    if cpu is not None:
        line["cpu_baseline"] = cpu
    ctx.close()
    if args.serving_requests > 0:
        line["serving"] = serving_block(args, rank, world)
    if rank == 0:
        print(json.dumps(line))


def serving_block(args, rank, world):
    """A short seeded serving stream after the stepper measurement (its
    context closed): the serving workload's Poisson arrivals, 2-D and 3-D
    solves of 50 RK4 steps adapted every 5 steps, each geometry served by
    its own host thread; p50/p99 time to solution and aggregate
    point-updates/s."""
    import torch
    from wabbit_gb300 import serving
    stream = serving.make_stream(args.serving_requests, rate=args.rate, seed=4 + rank)
    srv = serving.Server(budget_gb=args.budget_gb, chunk=5, adapt_every=5)
    srv.warm_up()
    torch.cuda.synchronize()
    recs, summ = srv.run(stream, realtime=True)
    srv.close()
    return {"requests": summ["requests"], "arrival_rate_per_s": args.rate, "steps_per_solve": 50,
            "adapt_every": 5, "value": sum_over_ranks(summ["point_updates"], world) / max_over_ranks(
                summ["wall_s"], world), "unit": "point-updates/s", "p50_s": summ["p50_s"], "p99_s": summ["p99_s"],
            "wall_s": summ["wall_s"], "phase_s": summ["phase_s"], "contexts_blocks": summ["workers"],
            "note": "time to solution = arrival to result on the host; IC generated on the device at admission "
                    "(inside the window); full stream: --workload serving --requests 256"}


def compare_plain(args, cfg, lv, co, u0, ids, masks, f, ctx, value, npts):
    """Plain per-solve FP64 path on the same grid and IC: one wg_rk4_step call
    per step, no graph. Also runs the measured configuration and the plain
    one for K steps from the same state and reports their relative L2
    difference (the FP64 path reproduces the oracle to 1e-12 per step)."""
    import torch
    from wabbit_gb300.solver import Context
    c64 = cfg.copy()
    c64.rhs_precision = 0
    ctx64 = Context(c64, len(lv) + 16)
    g = ctx64.forest()
    g.set_grid(lv, co)
    g.upload_interior(u0)
    if masks is not None and len(ids):
        g.set_mask_sparse(ids, masks)
    g.set_time(0.0)
    for _ in range(max(args.warmup, 1)):
        g.timeStep_tree()
    ctx64.synchronize()
    k = args.steps
    t0 = time.perf_counter()
    for _ in range(k):
        g.timeStep_tree()
    ctx64.synchronize()
    el = time.perf_counter() - t0
    v_plain = npts * k / el
    # accuracy: both from the IC for K steps
    g.upload_interior(u0)
    g.set_time(0.0)
    f.upload_interior(u0)
    f.set_time(0.0)
    for _ in range(k):
        g.timeStep_tree()
    f.run(k, use_graph=True)
    ctx.synchronize()
    a = f.download_interior()
    b = g.download_interior()
    err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    ctx64.close()
    return {"value": v_plain, "unit": "point-updates/s", "speedup": value / v_plain, "steps": k,
            "rel_l2_after_steps": err, "path": "FP64 strict-order-free fast stencils, wg_rk4_step per step, no graph"}


def run_serving(args, rank, world):
    """Serving workload: a seeded Poisson stream of independent solves
    (2-D and 3-D, 64-8192 blocks, 50 RK4 steps each, adapted every 5 steps:
    refine everywhere, 5 steps, adapt_tree with eps = 1e-3), admitted by HBM
    footprint and stepped in batched launches; aggregate point-updates/s
    with p50/p99 time to solution (arrival to result on the host)."""
    import torch
    from wabbit_gb300 import build, serving
    build.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    stream = serving.make_stream(args.requests, rate=args.rate, seed=4 + rank)
    srv = serving.Server(budget_gb=args.budget_gb, chunk=5, adapt_every=args.adapt_every)
    # warm-up: one small solve on every context (graph capture, autotuning)
    srv.warm_up()
    barrier(world)
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        recs, summ = srv.run(stream, realtime=True)
    srv.close()
    wall = max_over_ranks(summ["wall_s"], world)
    total = sum_over_ranks(summ["point_updates"], world)
    line = {
        "metric": "ACM point-updates/s/GPU", "value": total / wall, "unit": "point-updates/s", "n_gpus": world,
        "steps": 50, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 state, double-float (2xf32) stencils",
        "data": "synthetic (seeded Poisson stream, vortex ICs; see wabbit_gb300/serving.py)",
        "config": {"workload": "serving", "requests": args.requests, "arrival_rate_per_s": args.rate,
                   "budget_gb": args.budget_gb, "chunk_steps": 5, "arena_blocks": srv.capacity,
                   "adapt_every": args.adapt_every, "eps": srv.eps,
                   "cycle": "sync, refine everywhere, chunk of RK4 steps, adapt_tree" if args.adapt_every else None,
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "serving": {"p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "wall_s": summ["wall_s"],
                    "requests": summ["requests"], "point_updates": summ["point_updates"],
                    "phase_s": summ["phase_s"], "contexts_blocks": summ["workers"]},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def run_adapt(args, rank, world):
    """The adapt path at scale (configuration 5: 3-D CDF4,4, 99,184 blocks on
    five levels, eps = 1e-4 x Linfty norm): one step = adapt_tree on the
    whole tree (LIB/MESH/adapt_tree.f90:11-255) through wg_adapt: filtered
    ghost sync, full-tree FWT level by level with coarse extension and
    daughter-to-mother copies, indicator on the decomposition, security
    zone, flag consistency, deletion, reconstruction at the coarse/fine
    interfaces, pruning, final sync. Before every step the original grid and
    field are restored from a device copy of the interiors (untimed).
    value: input interior points per second of adapt_tree wall time."""
    import torch
    from wabbit_gb300 import build, workloads
    from wabbit_gb300.solver import Context, probe_alu
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    name = "adapt3d_cdf44"
    cfg = workloads.make_config(name)
    if args.jmax is not None:
        cfg.Jmax = args.jmax
    lv, co = workloads.make_grid(name, cfg)
    nblk = len(lv)
    npts = nblk * 16 ** 3
    u = workloads.adapt_field_device(cfg, lv, co)
    norms = u.abs().amax(dim=(0, 2, 3, 4)).cpu().numpy()
    eps_use = cfg.eps * norms
    # leaves + mothers of the full tree, plus a margin
    ctx = Context(cfg, int(nblk * 1.2) + 64)
    f = ctx.forest()
    stream = torch.cuda.ExternalStream(ctx.stream)

    def restore():
        f.set_grid(lv, co)
        f.upload_interior(u)
        torch.cuda.synchronize()

    def one(times=None):
        restore()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        t0 = time.perf_counter()
        ev[0].record(stream)
        n = f.adapt(eps_use)
        ev[1].record(stream)
        ev[1].synchronize()
        t1 = time.perf_counter()
        if times is not None:
            times["wall"] += t1 - t0
            times["device_tail"] += ev[0].elapsed_time(ev[1]) * 1e-3
        return n

    for _ in range(max(args.warmup, 1)):
        n_new = one()
    barrier(world)
    times = {"wall": 0.0, "device_tail": 0.0}
    with Clocks(local) as clk:
        for _ in range(args.steps):
            n_new = one(times)
    el = max_over_ranks(times["wall"], world)
    lv_new, _ = f.grid()
    # one more adapt with phase timing (stream synchronised at phase ends)
    f.adapt_profile(True)
    one()
    phases = f.adapt_profile(False)
    # the dominant kernels on the input grid, timed alone: FWT and IWT of every
    # leaf (one block component per CTA, FP64)
    restore()
    f.sync_ghosts_tree()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    f.wavelet_decompose()
    ev[1].record(stream)
    f.wavelet_reconstruct()
    ev[2].record(stream)
    ev[2].synchronize()
    fwt_ms, iwt_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    hbm_peak, hbm_src = measured_peaks()
    bytes_t = 2.0 * 8 * cfg.neq * npts          # read + write every interior value once
    # FP64 operations of the CDF4,4 FWT per block component: x pass on
    # Bs x (Bs+12)^2 points, y pass on Bs^2 x (Bs+12), z pass on Bs^3, half
    # SC (11 taps: 21 flops), half WC (5 taps: 9 flops)
    flops_fwt = nblk * cfg.neq * (16 * 28 * 28 + 16 * 16 * 28 + 16 ** 3) * 15.0
    fp64_peak, _ = probe_alu()
    line = {
        "metric": "adapt-path points/s/GPU", "value": sum_over_ranks(npts * args.steps / el, world),
        "unit": "points/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Fourier modes + tanh fronts; see wabbit_gb300/workloads.py)",
        "config": {"workload": name, "blocks": nblk, "points": npts, "levels": np.bincount(lv).tolist(),
                   "wavelet": "CDF44", "g": cfg.g, "Jmin": cfg.Jmin, "Jmax": cfg.Jmax, "eps": cfg.eps,
                   "eps_normalized": "Linfty",
                   "step": "adapt_tree (full-tree FWT with coarse extension, indicator, security zone, "
                           "gradedness, reconstruction at interfaces, final sync)",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "result": {"blocks_after": int(n_new), "levels_after": np.bincount(lv_new).tolist()},
        "adapt_phases_ms": phases,
        "kernels_ms_alone": {"fwt_all_leaves": fwt_ms, "iwt_all_leaves": iwt_ms},
        "roofline": {"bound": "hbm", "kernel": "tpo_kernel (FWT of every leaf)",
                     "achieved": bytes_t / (fwt_ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                     "frac": bytes_t / (fwt_ms * 1e-3) / 1e9 / hbm_peak, "traffic": None, "peak_source": hbm_src,
                     "algorithmic_bytes_per_launch": bytes_t},
        "roofline_alu": {"bound": "fp64", "achieved": flops_fwt / (fwt_ms * 1e-3) / 1e12,
                         "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": flops_fwt / (fwt_ms * 1e-3) / 1e12 / fp64_peak if fp64_peak else None,
                         "note": "FP64 FMA peak measured in this run; the FWT keeps the reference's separate "
                                 "multiplies and adds (no FMA), so half of it is its ceiling"},
        "clocks": clk.summary(),
    }
    del u
    torch.cuda.empty_cache()
    ctx.close()
    if not args.no_cpu and rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_adapt_sample(cfg)
    if rank == 0:
        print(json.dumps(line))


def cpu_adapt_sample(cfg, seconds=10.0):
    """The oracle's adapt_tree (lifted, single thread) on the same workload at
    Jmax=4 (a bounded sample of the same kind of grid and field), repeated for
    about `seconds`; points per second of input interior."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from wabbit_gb300 import workloads
    import pyoracle
    c = workloads.make_config("adapt3d_cdf44")
    c.Jmax = 4
    lv, co = workloads.make_grid("adapt3d_cdf44", c)
    u = workloads.adapt_field_device(c, lv, co).cpu().numpy()
    norms = np.abs(u).max(axis=(0, 2, 3, 4))
    full = pyoracle.pad_blocks(c, u)
    done, t = 0, 0.0
    while t < seconds:
        o = pyoracle.Oracle(c)
        o.set_grid(lv, co, full)
        t0 = time.perf_counter()
        o.sync(c.g, c.g, ignore_filter=False)
        o.adapt(c.eps * norms)
        t += time.perf_counter() - t0
        done += 1
    return {"value": done * len(lv) * 16 ** 3 / t, "unit": "points/s", "cores": 1, "kind": "port",
            "sample": f"adapt3d_cdf44 at Jmax=4 ({len(lv)} blocks), {done} adapt_tree passes in {t:.1f} s"}


def run_adapt_loop(args, rank, world):
    """Configuration 1: 2-D ACM (Bs=16, g=4, CDF4,0, Jmin=2, Jmax=5, eps=1e-3
    absolute) with the grid adapted every step. The initial grid comes from
    the vortex IC on the equidistant Jmax grid, adapted until it no longer
    changes (adapt_inicond). One step = ghost sync, refine everywhere, one
    RK4 step, adapt (LIB/MAIN/main.f90:314-400). value: point-updates/s of
    the RK4 steps over the wall time of the whole loop (fused); the stepper
    alone and the adapt part are reported beside it."""
    import torch
    from wabbit_gb300 import build, grids, workloads
    from wabbit_gb300.solver import Context
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cfg = workloads.make_config("acm2d_vortex")
    lv, co = grids.equidistant(2, cfg.Jmax)
    eps = np.full(cfg.neq, cfg.eps)
    ctx = Context(cfg, 8 * len(lv))
    f = ctx.forest()
    f.set_grid(lv, co)
    f.upload_interior(workloads.initial_condition("acm2d_vortex", cfg, lv, co))
    n_prev = -1
    while n_prev != f.nblocks:
        n_prev = f.nblocks
        f.adapt(eps)
    f.set_time(0.0)
    npts_blk = 16 * 16

    def one(times=None):
        t0 = time.perf_counter()
        f.sync_ghosts_tree()
        f.refine_everywhere()
        t1 = time.perf_counter()
        n = f.nblocks
        f.timeStep_tree()
        t2 = time.perf_counter()
        f.adapt(eps)
        t3 = time.perf_counter()
        if times is not None:
            times["refine"] += t1 - t0
            times["step"] += t2 - t1
            times["adapt"] += t3 - t2
            times["points"] += n * npts_blk
        return n

    for _ in range(max(args.warmup, 1)):
        one()
    barrier(world)
    times = {"refine": 0.0, "step": 0.0, "adapt": 0.0, "points": 0}
    blocks = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            blocks.append(one(times))
        el = max_over_ranks(time.perf_counter() - t0, world)
    t_end, dt_last = f.time()
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        cpu = cpu_adapt_loop(cfg, lv, co, eps)
    line = {
        "metric": "ACM point-updates/s/GPU", "value": sum_over_ranks(times["points"] / el, world),
        "unit": "point-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Gaussian vortices; see wabbit_gb300/workloads.py)",
        "config": {"workload": "acm2d_vortex_adapt", "dim": 2, "Bs": [16, 16], "g": cfg.g, "wavelet": "CDF40",
                   "Jmin": cfg.Jmin, "Jmax": cfg.Jmax, "eps": cfg.eps, "eps_normalized": False,
                   "blocks_min": int(min(blocks)), "blocks_max": int(max(blocks)),
                   "step": "sync g, refine everywhere, RK4 (FP64 fast), adapt",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "stepper_only": {"value": times["points"] / times["step"], "unit": "point-updates/s"},
        "phase_ms_per_step": {k: 1e3 * times[k] / args.steps for k in ("refine", "step", "adapt")},
        "clocks": clk.summary(), "t_end": t_end,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def cpu_adapt_loop(cfg, lv, co, eps, seconds=12.0):
    """The oracle running the same adapt loop (all host cores) for a bounded
    time, from the same adapted initial grid."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from wabbit_gb300 import workloads
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(cfg, threads=threads)
    u = workloads.initial_condition("acm2d_vortex", cfg, lv, co)
    o.set_grid(lv, co, pyoracle.pad_blocks(cfg, u[:, :, 0]))
    n_prev = -1
    while n_prev != o.nblocks:
        n_prev = o.nblocks
        o.adapt(eps)
    t = 0.0
    points = 0
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds and steps < 50:
        o.sync(cfg.g, cfg.g, ignore_filter=True)
        o.refine_everywhere()
        points += o.nblocks * 256
        t, _ = o.step(t)
        o.adapt(eps)
        steps += 1
    el = time.perf_counter() - t0
    return {"value": points / el, "unit": "point-updates/s", "cores": threads, "kind": "port",
            "sample": f"acm2d_vortex_adapt, {steps} steps of the same loop in {el:.1f} s"}


def capi_graph_kernels(ctx):
    from wabbit_gb300 import capi
    n = ctx.L.wg_graph_kernels(ctx.h)
    return int(capi.check(n))


# the reference's own logged rate: TESTING/acm/3vortices/3vorticesEquiFD4_CDF40/
# log.original.txt, "TOPLEVEL: time stepper" 2.630 s for the 3073 RK4 steps
# (t = 10 -> 20) of 64 blocks of 32^2 points on 12 MPI ranks
REF_LOG = {"value": 3073 * 64 * 32 * 32 / 2.630, "unit": "point-updates/s", "ranks": 12,
           "case": "3vorticesEquiFD4_CDF40: 2-D, 64 blocks of 32^2, CDF40, FD4 skew-symmetric, RK4",
           "source": "TESTING/acm/3vortices/3vorticesEquiFD4_CDF40/log.original.txt, TOPLEVEL: time stepper "
                     "2.630 s over 3073 steps"}


def oracle_on_log_case(threads, steps=400):
    """The oracle on the case of the reference's log (the committed t = 10
    state of 3vorticesEquiFD4_CDF40), point-updates/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from wabbit_gb300 import config
    z = np.load(os.path.join(ROOT, "tests", "golden", "vortex2d_equi.npz"))
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
    o = pyoracle.Oracle(c, threads=threads)
    o.set_grid(z["level"], z["coords"], None)
    o.set_interior(z["u_in"])
    t = float(z["t_in"])
    t, _ = o.step(t)
    t0 = time.perf_counter()
    for _ in range(steps):
        t, _ = o.step(t)
    return 64 * 32 * 32 * steps / (time.perf_counter() - t0)


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path: the oracle (the
    reference is Fortran and no Fortran compiler exists in this image; the
    oracle reproduces the reference's regression outputs bit for bit) on the
    same workload as the GPU arm -- grid, IC, mask -- with every host core,
    W warm-up and K timed RK4 steps of the whole grid. If the host cannot
    hold the workload, the largest Jmax that fits is used and the line says
    so."""
    if rank != 0:
        return
    from wabbit_gb300 import workloads
    cores = os.cpu_count() or 1
    jmax_full = args.jmax if args.jmax is not None else workloads.make_config(args.workload).Jmax
    jmax = jmax_full
    avail = host_mem_available()
    while avail is not None and jmax > 4 and oracle_bytes(args.workload, jmax) > 0.8 * avail:
        jmax -= 1
    o, npts, cfg, nblk = oracle_for(args.workload, jmax=jmax, threads=cores)
    t = 0.0
    for _ in range(args.warmup):
        t, _ = o.step(t)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t, _ = o.step(t)
    el = time.perf_counter() - t0
    del o
    value = npts * args.steps / el
    same = jmax == jmax_full
    sample = (f"{args.workload} at Jmax={jmax} ({nblk} blocks, {npts} points, same grid, IC and mask as the GPU "
              f"arm{'' if same else '; the full grid does not fit into host memory'}), {args.steps} RK4 steps of "
              f"the whole grid per run, {cores} threads")
    # one core, and the oracle on the case of the reference's own log
    o1, npts1, _, nblk1 = oracle_for(args.workload, jmax=4, threads=1)
    steps1, el1 = time_oracle(o1, 50, 1, 6.0)
    del o1
    log_all = oracle_on_log_case(cores)
    log_12 = oracle_on_log_case(min(12, cores))
    line = {
        "metric": "ACM point-updates/s/GPU", "value": value, "unit": "point-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded IC and grid, see wabbit_gb300/workloads.py)",
        "config": {"workload": args.workload, "Jmax": jmax, "blocks": nblk, "points": npts, "same_config": same,
                   "sample": sample},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "point-updates/s", "cores": cores, "kind": "port",
                         "sample": sample, "one_core_value": npts1 * steps1 / el1,
                         "one_core_sample": f"Jmax=4 grid ({nblk1} blocks), {steps1} RK4 steps in {el1:.1f} s",
                         "build": "g++ -O3 -ffp-contract=off -fopenmp (oracle/Makefile)"},
        "e2e": {"value": value, "unit": "point-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_log": dict(REF_LOG, oracle_same_case={f"{cores}_threads": log_all,
                                                         f"{min(12, cores)}_threads": log_12}),
        "note": "the reference is Fortran (no Fortran compiler in this image); the timed path is the oracle, "
                "its bit-exact C++ restatement, labelled a CPU restatement, not the reference binary",
    }
    print(json.dumps(line))


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.traffic_case:
        run_traffic_case(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "serving":
        run_serving(args, rank, world)
    elif args.workload == "adapt3d_cdf44":
        run_adapt(args, rank, world)
    elif args.workload == "acm2d_vortex_adapt":
        run_adapt_loop(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
