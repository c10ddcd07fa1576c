#!/usr/bin/env python
"""Benchmark of the BEM operator apply (KIFMM matvec) on GB300.

Workload (the elastic fault case): a planar 2 x 2 fault dipping 45 degrees,
a 128 x 128 quad grid split into 32,768 triangles, 3 Gauss points each
(98,304 points, obs = src), Kelvin elastic displacement AND traction kernels
(shear modulus 1, Poisson ratio 0.25), slip = uniform[-1,1] x cosine taper
(seed 1).  FMM: order 296 requested translation-surface points (295 used;
"order 8" read as 6 (p-1)^2 + 2), MAC 0.3, 64 points per leaf, d = 0.05.

One step = one apply of the displacement operator and one of the traction
operator to the slip (2 x 98,304 points x RHS).  ``value`` is whole-job
points*RHS/s of the precision (mixed) form with inputs resident in HBM;
``e2e`` is the same through the public C ABI with host buffers (the host to
device copy of the slip and the device to host copy of the result are inside
the timed region).  L2 is flushed (256 MB written) before every timed step,
outside the step's timing: the per-leaf L2P operators (0.3 GB per kernel) are
larger than the 129 MB L2, but the M2L operator planes (42 MB per kernel)
alone would stay resident.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With --gpus N > 1 (under torchrun) every rank runs an independent replica of
the workload (the apply does not shard across GPUs: replicas only).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "3bem_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "FMM BEM matvec points*RHS/sec @1e-6 rel err: mixed-prec batched vs plain FP64"
MU, NU = 1.0, 0.25
ORDER, MAC, LEAF, D = 296, 0.3, 64, 0.05
N_GRID = 128
N_ERR_ROWS = 4096



def setup_phases(ops):
    """Construction phase seconds summed over the operators (FMMOperator.setup_times)."""
    out = {}
    for op in ops:
        for name, sec in op.setup_times():
            out[name] = round(out.get(name, 0.0) + sec, 4)
    return out

def workload(grid=N_GRID):
    from tbempy import meshes
    locs, nrm, w, uv = meshes.fault_points(grid, 45.0)
    x = meshes.tapered_slip(uv, seed=1)
    return locs, nrm, w, x


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def aggregate(seconds, units_per_rank, dist=None, device=None):
    """Whole-job throughput of independent replicas: every rank processed
    `units_per_rank`; the job took the slowest rank's time."""
    world = 1
    if dist is not None and dist.is_initialized():
        import torch
        world = dist.get_world_size()
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return world * units_per_rank / seconds, seconds


def m2l_flops(op, n_rhs):
    """M2L flops of one apply.

    reference: the reference formulation's count, one dense (R n_s) x (R n_s)
    product per M2L pair and right-hand side (2 flops per entry);
    tensor: what the compressed form's tensor-core kernel executes, one
    r_out x r_in product per pair and right-hand side, each as six bf16
    products (the three-term split), 2 flops per multiply-add."""
    n = op.n_surface() * op.R
    pairs = len(op.list("m2l")[0])
    ri, ro = op.m2l_ranks()
    return {"reference": 2.0 * n * n * pairs * n_rhs,
            "tensor": 6 * 2.0 * ri * ro * pairs * n_rhs if ri else None,
            "pairs": pairs}


def cpu_operators(locs, nrm, w, threads):
    """The oracle (CPU restatement of the reference FMM, OpenMP) built on the
    same workload, both kernels.  Returns (operators, setup seconds, threads)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    ops = [oracle.OracleFMM(name, locs, nrm, locs, nrm, w, MAC, ORDER, LEAF, D, False, MU, NU)
           for name in ("ElasticDisplacement", "ElasticTraction")]
    return ops, time.perf_counter() - t0, oracle.max_threads()


def cpu_apply_seconds(ops, x, fraction):
    """One step of the oracle operators timed on a bounded sample: the leading
    `fraction` of every task list, extrapolated to a full apply."""
    total = 0.0
    for o in ops:
        t0 = time.perf_counter()
        o.apply(x, list_fraction=fraction)
        total += (time.perf_counter() - t0) / fraction
    return total


def cpu_calibration(ops, x, fraction):
    """One FULL oracle apply of the first operator (the displacement kernel)
    against its sampled, extrapolated time: the ratio full / sampled that
    corrects the extrapolation of every sampled step."""
    t0 = time.perf_counter()
    ops[0].apply(x, list_fraction=fraction)
    sampled = (time.perf_counter() - t0) / fraction
    t0 = time.perf_counter()
    ops[0].apply(x)
    full = time.perf_counter() - t0
    return {"full_apply_s": full, "sampled_extrapolated_s": sampled, "ratio": full / sampled,
            "operator": "ElasticDisplacement", "fraction": fraction}


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the host cores (the oracle
    port; the reference's own build needs its checkout, which does not travel
    with this repository)."""
    if rank != 0:
        return
    locs, nrm, w, x = workload()
    threads = os.cpu_count() or 1
    frac = args.cpu_fraction
    # built once, like the operator of the GPU arm; each step is one apply
    ops, setup, cores = cpu_operators(locs, nrm, w, threads)
    calib = cpu_calibration(ops, x, frac)
    samples = []
    for i in range(args.warmup + args.steps):
        t_full = cpu_apply_seconds(ops, x, frac) * calib["ratio"]
        if i >= args.warmup:
            samples.append(t_full)
    t = float(np.median(samples))
    value = 2 * len(locs) / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "points*RHS/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded dipping-fault mesh)",
        "config": config_dict(1),
        "cpu_baseline": {"value": value, "unit": "points*RHS/s", "cores": cores, "kind": "port",
                         "sample": "leading %.3g of every FMM task list per step, both kernels, "
                                   "extrapolated to a full apply and scaled by the measured "
                                   "full / sampled ratio of one full displacement apply" % frac,
                         "calibration": calib},
        "e2e": {"value": value, "unit": "points*RHS/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "setup_s": setup,
    }
    print(json.dumps(line), flush=True)


def config_dict(n_rhs):
    return {"workload": "elastic fault: Kelvin displacement + traction FMM apply, 98,304 points "
                        "(128x128 quads x 2 tris x 3 Gauss pts), dip 45 deg",
            "kernels": ["ElasticDisplacement", "ElasticTraction"],
            "fmm": {"order_requested": ORDER, "surface_points": 295, "mac": MAC,
                    "min_pts_per_cell": LEAF, "d": D, "account_for_small_cells": False},
            "n_points": 3 * 2 * N_GRID * N_GRID, "n_rhs": n_rhs,
            "precision": "mixed: far field in the M2L SVD bases (FP32), M2L products on "
                         "tcgen05 3xBF16, P2P FP32 compensated",
            "step": "one displacement apply and one traction apply, replayed as one CUDA graph "
                    "with the two applies in parallel branches (tbem_fmm_graph_launch); "
                    "ms_per_step_sequential: the same applies one after the other",
            "l2": "flushed before every timed step (256 MB write, outside the step timing)"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the tensor-core M2L kernel on the default workload, from a one-pass ncu
# capture of this bench (ncu --metrics dram__bytes_read.sum,
# dram__bytes_write.sum --clock-control none -k regex:tc_gemm -s 40 -c 1
# python bench.py --steps 2 --warmup 3 --no-cpu --no-plain)
M2L_TC_DRAM_BYTES = 59.53e6


def _events_ms(torch, fn, steps, stream, flush=None):
    """Mean device milliseconds of fn over `steps` runs, CUDA events on the
    stream the work is issued to (L2 flushed before each when given)."""
    pairs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
             for _ in range(steps)]
    for e0, e1 in pairs:
        if flush is not None:
            flush.fill_(1)
        e0.record(stream)
        fn()
        e1.record(stream)
    torch.cuda.synchronize()
    return sum(e0.elapsed_time(e1) for e0, e1 in pairs) / steps


def _phases(op, fn):
    """Per-phase milliseconds of one run of fn (events between the passes)."""
    op.phase_times()
    op.set_timing(True)
    fn()
    ph = dict(op.phase_times())
    op.set_timing(False)
    return ph


# ---------------------------------------------------------------- sphere workload

SPHERE_ORDER, SPHERE_LEAF = 152, 50


def sphere_workload():
    """The plain FP64 Laplace single-layer workload: icosahedron subdivided 4
    times (5,120 triangles, radius 1), 3 Gauss points per triangle (15,360
    points), weights area / 3, outward normals, density uniform[-1, 1] seed 0."""
    from tbempy import meshes
    locs, nrm, w = meshes.sphere_points(4)
    x = np.random.default_rng(0).uniform(-1, 1, len(locs))
    return locs, nrm, w, x


def sphere_config():
    return {"workload": "Laplace single layer 1/(4 pi r) FMM apply, 15,360 points (icosahedron "
                        "subdivided 4 times, 3 Gauss points per triangle), 1 RHS",
            "kernel": "LaplaceSingle",
            "fmm": {"order_requested": SPHERE_ORDER, "surface_points": 152, "mac": MAC,
                    "min_pts_per_cell": SPHERE_LEAF, "d": D, "account_for_small_cells": False},
            "n_points": 15360, "n_rhs": 1,
            "precision": "plain FP64 (the reference's formulation)",
            "l2": "flushed before every timed step (256 MB write, outside the step timing)"}


def run_sphere(args, rank, world, local):
    from oracle import oracle
    if args.impl == "reference":
        if rank != 0:
            return
        locs, nrm, w, x = sphere_workload()
        threads = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
        oracle.build()
        t0 = time.perf_counter()
        o = oracle.OracleFMM("LaplaceSingle", locs, nrm, locs, nrm, w, MAC, SPHERE_ORDER, SPHERE_LEAF, D)
        setup = time.perf_counter() - t0
        ts = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            o.apply(x)
            if i >= args.warmup:
                ts.append(time.perf_counter() - t0)
        t = float(np.median(ts))
        value = len(locs) / t
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "points*RHS/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded icosphere)", "config": sphere_config(),
            "cpu_baseline": {"value": value, "unit": "points*RHS/s", "cores": oracle.max_threads(),
                             "kind": "port", "sample": "one full oracle FMM apply per step"},
            "e2e": {"value": value, "unit": "points*RHS/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "setup_s": setup}), flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    from tbempy import ThreeD
    from tbempy import _lib
    import ctypes as C
    locs, nrm, w, x = sphere_workload()
    N = len(locs)
    K = ThreeD.LaplaceSingle()
    cfg = ThreeD.FMMConfig(MAC, SPHERE_ORDER, SPHERE_LEAF, D, False)
    t0 = time.perf_counter()
    op = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64", device=local)
    setup_s = time.perf_counter() - t0
    opm = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", device=local)
    xd = torch.tensor(x, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        op.apply(xd)
        opm.apply(xd)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = _events_ms(torch, lambda: op.apply(xd), args.steps, stream, flush)
        ms_mixed = _events_ms(torch, lambda: opm.apply(xd), args.steps, stream, flush)
    launches = op.last_launches() * args.steps
    phases = _phases(op, lambda: op.apply(xd))
    phases_mixed = _phases(opm, lambda: opm.apply(xd))
    # end to end through the C ABI, pinned host buffers
    xh = torch.tensor(x).pin_memory()
    yh = torch.empty(N, dtype=torch.float64).pin_memory()
    L = _lib.lib()
    for _ in range(2):
        _lib.check(L.tbem_fmm_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 1, None))
    e2e = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(L.tbem_fmm_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 1, None))
        e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e))
    y = yh.numpy().copy()
    exact = ThreeD.DirectOperator(K, locs, nrm, locs, nrm, w).apply(x)
    err = float(np.linalg.norm(y - exact) / np.linalg.norm(exact))
    ym = opm.apply(x)
    err_m = float(np.linalg.norm(ym - exact) / np.linalg.norm(exact))
    parity = None
    fx = os.path.join(ROOT, "tests", "golden", "fmm_laps_icosphere15k.npz")
    if os.path.exists(fx):
        g = np.load(fx)
        own = float(np.linalg.norm(y - g["y_ref"]) / np.linalg.norm(g["y_ref"]))
        for which in (0, 1):
            for lev, m in enumerate(g["c2e%d" % which]):
                op.set_c2e(which, lev, m)
        yr = op.apply(x)
        parity = {"own_operators_vs_reference": own,
                  "reference_operators_vs_reference": float(np.linalg.norm(yr - g["y_ref"]) /
                                                            np.linalg.norm(g["y_ref"])),
                  "reference_ulp_floor": float(g["ulp_floor"])}
    # roofline: the plain form's M2L products (FP64 grouped GEMM over the
    # deduplicated operators), 2 n^2 flops per pair
    n = op.n_surface()
    pairs = len(op.list("m2l")[0])
    m2l_ms = phases.get("m2l", float("nan"))
    achieved = 2.0 * n * n * pairs / (m2l_ms / 1e3) / 1e12
    fp64_peak = ThreeD.fma_peak_tflops(True, local)
    cpu = None
    if not args.no_cpu:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        oracle.build()
        o = oracle.OracleFMM("LaplaceSingle", locs, nrm, locs, nrm, w, MAC, SPHERE_ORDER, SPHERE_LEAF, D)
        t0 = time.perf_counter()
        o.apply(x)
        tc = time.perf_counter() - t0
        cpu = {"value": N / tc, "unit": "points*RHS/s", "cores": oracle.max_threads(), "kind": "port",
               "sample": "one full oracle FMM apply (%.2f s)" % tc}
    print(json.dumps({
        "metric": METRIC, "value": N / (ms / 1e3), "unit": "points*RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded icosphere)", "config": sphere_config(), "clocks": clk.summary(),
        "e2e": {"value": N / e2e_s, "unit": "points*RHS/s", "h2d_bytes_per_step": 8 * N,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": launches,
        "roofline": {"bound": "fp64", "kernel": "grouped_gemm_kernel<double>: M2L products",
                     "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp64_peak,
                     "peak_kind": "measured FP64 FMA rate (tbem_fma_peak microbenchmark)",
                     "traffic": None, "flops_per_launch": 2.0 * n * n * pairs, "launch_ms": m2l_ms},
        "phases_ms": phases, "rel_err_vs_direct": err, "parity": parity,
        "precision_form": {"ms_per_step": ms_mixed, "points_rhs_per_s": N / (ms_mixed / 1e3),
                           "rel_err_vs_direct": err_m, "phases_ms": phases_mixed,
                           "speedup_vs_plain": ms / ms_mixed},
        "cpu_baseline": cpu, "setup_s": setup_s, "setup_phases_s": setup_phases([op])}), flush=True)


# --------------------------------------------------------------- batched workload

BATCH_ORDER, BATCH_LEAF = 152, 128


def batched_config(n_meshes, n_rhs, n_points):
    return {"workload": "Laplace double layer FMM apply on %d icospheres (subdivision 2..6, "
                        "radius lognormal(0, 0.5), centres in [-100, 100]^3, 3 Gauss points per "
                        "triangle), %d right-hand sides, one operator" % (n_meshes, n_rhs),
            "kernel": "LaplaceDouble", "n_meshes": n_meshes, "n_points": n_points, "n_rhs": n_rhs,
            "fmm": {"order_requested": BATCH_ORDER, "surface_points": 152, "mac": MAC,
                    "min_pts_per_cell": BATCH_LEAF, "d": D, "account_for_small_cells": False},
            "precision": "mixed: far field in the M2L SVD bases (FP32), M2L products on tcgen05 "
                         "3xBF16, P2P FP32 compensated; every mesh in the cube [-1,1]^3 of its own",
            "launch": "the whole apply captured in one CUDA graph, replayed once per step",
            "l2": "inputs (%.1f GB) larger than L2; no flush" % (8.0 * n_points * n_rhs / 1e9)}


def _batched_cpu_seconds(locs, nrm, w, off, n_rhs):
    """The reference's way: one operator per mesh, one right-hand side per
    apply (the oracle port, all host threads).  One mesh per subdivision
    level is timed -- levels 2-4 with a full apply, levels 5-6 on the leading
    fraction of every task list, extrapolated -- and the batch's time is
    the sum over meshes of their level's time, times n_rhs.  Level 4 is also
    timed sampled, to state the extrapolation's error."""
    from oracle import oracle
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    oracle.build()
    sizes = np.diff(off)
    per_size, detail = {}, {}
    rng = np.random.default_rng(0)
    for n in sorted(set(sizes.tolist())):
        m = int(np.nonzero(sizes == n)[0][0])
        sl = slice(off[m], off[m + 1])
        o = oracle.OracleFMM("LaplaceDouble", locs[sl], nrm[sl], locs[sl], nrm[sl], w[sl], MAC,
                             BATCH_ORDER, BATCH_LEAF, D)
        x = rng.uniform(-1, 1, n)
        frac = 1.0 if n <= 15360 else (0.1 if n <= 61440 else 0.02)
        t0 = time.perf_counter()
        o.apply(x, list_fraction=frac)
        t = (time.perf_counter() - t0) / frac
        per_size[n] = t
        detail[str(n)] = {"seconds_per_apply": t, "list_fraction": frac}
        if n == 15360:
            t0 = time.perf_counter()
            o.apply(x, list_fraction=0.1)
            ts = (time.perf_counter() - t0) / 0.1
            detail["extrapolation_check"] = {"points": n, "full_s": t, "sampled_0.1_s": ts,
                                             "ratio": ts / t}
        del o
    total = sum(per_size[int(n)] for n in sizes) * n_rhs
    return total, detail, oracle.max_threads()


def run_batched(args, rank, world, local):
    from tbempy import meshes
    locs, nrm, w, off, X = meshes.sphere_batch(n_meshes=args.meshes, seed=2, n_rhs=args.batch_rhs)
    N, B = len(locs), X.shape[0]
    if args.impl == "reference":
        if rank != 0:
            return
        t, detail, cores = _batched_cpu_seconds(locs, nrm, w, off, B)
        value = N * B / t
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "points*RHS/s",
            "n_gpus": world, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded icospheres)", "config": batched_config(len(off) - 1, B, N),
            "cpu_baseline": {"value": value, "unit": "points*RHS/s", "cores": cores, "kind": "port",
                             "sample": "one mesh per subdivision level timed (levels 5-6 on a "
                                       "fraction of the task lists), summed over the meshes, "
                                       "one RHS per apply", "detail": detail},
            "e2e": {"value": value, "unit": "points*RHS/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    import ctypes as C
    torch.cuda.set_device(local)
    from tbempy import ThreeD
    from tbempy import _lib
    K = ThreeD.LaplaceDouble()
    cfg = ThreeD.FMMConfig(MAC, BATCH_ORDER, BATCH_LEAF, D, False)
    t0 = time.perf_counter()
    op = ThreeD.BatchedFMMOperator(K, locs, nrm, w, off, cfg, precision="mixed", device=local)
    setup_s = time.perf_counter() - t0
    xd = torch.tensor(X, device="cuda")
    yd = torch.empty_like(xd)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream if stream.cuda_stream else 1)
    t0 = time.perf_counter()
    graph = ThreeD.FMMGraph([op], [xd], [yd], n_rhs=B)  # runs one apply, then captures one
    graph_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        graph.launch(sp)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = _events_ms(torch, lambda: graph.launch(sp), args.steps, stream)
    launches = op.last_launches() * args.steps
    phases = _phases(op, lambda: op.apply(xd))
    # end to end through the C ABI, pinned host buffers
    xh = torch.tensor(X).pin_memory()
    yh = torch.empty((B, N), dtype=torch.float64).pin_memory()
    L = _lib.lib()
    _lib.check(L.tbem_fmm_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), B, None))
    e2e = []
    for _ in range(max(2, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(L.tbem_fmm_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), B, None))
        e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e))
    Y = yh.numpy()
    # accuracy: every mesh against the FP64 direct sum on up to 128 sampled rows
    rng = np.random.default_rng(7)
    errs = []
    rows_of = []
    for m in range(len(off) - 1):
        sl = slice(off[m], off[m + 1])
        rows = np.sort(rng.choice(off[m + 1] - off[m], min(128, off[m + 1] - off[m]), replace=False))
        rows_of.append(rows)
        d = ThreeD.DirectOperator(K, locs[sl][rows], nrm[sl][rows], locs[sl], nrm[sl], w[sl])
        ex = d.apply(np.ascontiguousarray(X[:, sl]))
        got = Y[:, off[m] + rows]
        errs.append(float(np.linalg.norm(got - ex) / np.linalg.norm(ex)))
    # roofline: the M2L products on the tensor cores (one launch per RHS chunk)
    ri, ro = op.m2l_ranks()
    pairs = len(op.list("m2l")[0])
    m2l_ms = phases.get("m2l", float("nan"))
    hbm, bf16, peak_kind = peaks()
    flops = 6 * 2.0 * ri * ro * pairs * B
    achieved = flops / (m2l_ms / 1e3) / 1e12
    del xh, yh
    # the plain FP64 form on the same meshes, one right-hand side
    plain = None
    if not args.no_plain:
        t0 = time.perf_counter()
        pop = ThreeD.BatchedFMMOperator(K, locs, nrm, w, off, cfg, precision="fp64", device=local)
        psetup = time.perf_counter() - t0
        x0 = torch.tensor(X[0], device="cuda")
        pop.apply(x0)
        pms = _events_ms(torch, lambda: pop.apply(x0), 1, stream)
        y0 = pop.apply(X[0])
        perr = []
        for m in range(len(off) - 1):
            sl = slice(off[m], off[m + 1])
            rows = rows_of[m]
            d = ThreeD.DirectOperator(K, locs[sl][rows], nrm[sl][rows], locs[sl], nrm[sl], w[sl])
            ex = d.apply(np.ascontiguousarray(X[0, sl]))
            perr.append(float(np.linalg.norm(y0[off[m] + rows] - ex) / np.linalg.norm(ex)))
        plain = {"ms_per_apply_1rhs": pms, "points_rhs_per_s": N / (pms / 1e3), "setup_s": psetup,
                 "rel_err_vs_direct_max": max(perr),
                 "speedup_mixed_batched_vs_plain": (N * B / (ms / 1e3)) / (N / (pms / 1e3))}
        del pop
    cpu = None
    if not args.no_cpu:
        t, detail, cores = _batched_cpu_seconds(locs, nrm, w, off, B)
        cpu = {"value": N * B / t, "unit": "points*RHS/s", "cores": cores, "kind": "port",
               "sample": "one mesh per subdivision level timed (levels 5-6 on a fraction of the "
                         "task lists), summed over the meshes, one RHS per apply",
               "detail": detail}
    print(json.dumps({
        "metric": METRIC, "value": N * B / (ms / 1e3), "unit": "points*RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded icospheres)", "config": batched_config(len(off) - 1, B, N),
        "clocks": clk.summary(),
        "e2e": {"value": N * B / e2e_s, "unit": "points*RHS/s", "h2d_bytes_per_step": 8 * N * B,
                "d2h_bytes_per_step": 8 * N * B},
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "kernel": "tc_gemm_kernel: compressed M2L products, tcgen05 3xBF16",
                     "achieved": achieved, "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
                     "peak_kind": peak_kind + " bf16 dense (burst)", "traffic": None,
                     "flops_per_apply": flops, "m2l_ms_per_apply": m2l_ms},
        "phases_ms": phases, "m2l_ranks": [ri, ro], "m2l_pairs": pairs,
        "rel_err_vs_direct": {"max_over_meshes": max(errs), "median": float(np.median(errs)),
                              "rows_per_mesh": 128},
        "plain_fp64": plain, "cpu_baseline": cpu, "setup_s": setup_s,
        "setup_phases_s": setup_phases([op]), "graph_capture_s": graph_s,
        }), flush=True)


def misfit_config():
    return {"workload": "differentiated misfit L = 0.5 ||G s - d||^2, elastic displacement, "
                        "64 x 64-quad bumpy fault (24,576 points) -> 16,384 observers on z = 0",
            "kernel": "ElasticDisplacement", "n_src": 24576, "n_obs": 16384, "n_rhs": 1,
            "fmm": {"order_requested": ORDER, "surface_points": 295, "mac": MAC,
                    "min_pts_per_cell": LEAF, "d": D, "account_for_small_cells": False},
            "step": "one gradient dL/ds: a forward apply and a transposed apply (value counts "
                    "the observation points of the forward apply)",
            "precision": "mixed (both trees cut from one cube: compressed tensor-core M2L)",
            "l2": "flushed before every timed step (256 MB write, outside the step timing)"}


def run_misfit(args, rank, world, local):
    from tbempy import meshes
    v, t, obs, on, s_np, s2_np, noise = meshes.misfit_workload()
    sl, sn, sw = meshes.points_from_mesh(v, t)
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        oracle.build()
        o = oracle.OracleFMM("ElasticDisplacement", obs, on, sl, sn, sw, MAC, ORDER, LEAF, D)
        frac = args.cpu_fraction * 10
        ts = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            o.apply(s_np, list_fraction=frac)
            if i >= args.warmup:
                ts.append((time.perf_counter() - t0) / frac)
        tt = float(np.median(ts))
        value = len(obs) / tt
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "points*RHS/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded bumpy fault)", "config": misfit_config(),
            "cpu_baseline": {"value": value, "unit": "points*RHS/s", "cores": oracle.max_threads(),
                             "kind": "port", "sample": "forward oracle apply on the leading %.2g of "
                                                       "every task list, extrapolated (the reference "
                                                       "has no transposed apply)" % frac},
            "e2e": {"value": value, "unit": "points*RHS/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    from tbempy import ThreeD, autograd
    K = ThreeD.ElasticDisplacement(MU, NU)
    Dop = ThreeD.DirectOperator(K, obs, on, sl, sn, sw)
    d = torch.tensor(Dop.apply(s2_np) + noise, device="cuda")
    s = torch.tensor(s_np, device="cuda")
    t0 = time.perf_counter()
    op = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, ThreeD.FMMConfig(MAC, ORDER, LEAF, D, False),
                            precision="mixed", device=local)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")

    def grad_step():
        r = op.apply(s) - d
        return op.apply_adjoint(r)

    for _ in range(args.warmup):
        grad_step()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = _events_ms(torch, grad_step, args.steps, stream, flush)
        ms_fwd = _events_ms(torch, lambda: op.apply(s), args.steps, stream, flush)
    phases = _phases(op, lambda: op.apply(s))
    # the vertex-coordinate gradient: the FMM's source gradients (transposed
    # passes with the kernel's derivatives) through torch's chain rule from the
    # vertices to the points, normals and weights; the direct kernel-gradient
    # pass (O(N M)) beside it as the check
    V = torch.tensor(v, device="cuda", requires_grad=True)
    OL, ON = torch.tensor(obs, device="cuda"), torch.tensor(on, device="cuda")

    def vertex_grad(use_fmm):
        V.grad = None
        a, b, c = meshes.points_from_mesh_torch(V, t)
        y = (autograd.fmm_apply_sources(op, a, b, c, s) if use_fmm
             else autograd.direct_apply(K, OL, ON, a, b, c, s))
        (0.5 * ((y - d) ** 2).sum()).backward()

    vertex_grad(True)
    gv_fmm = V.grad.clone()
    ms_vert = _events_ms(torch, lambda: vertex_grad(True), args.steps, stream)
    vertex_grad(False)
    gv_dir = V.grad.clone()
    ms_vert_direct = _events_ms(torch, lambda: vertex_grad(False), 1, stream)
    err_vert = float(torch.linalg.norm(gv_fmm - gv_dir) / torch.linalg.norm(gv_dir))
    # the observers' position gradient of the same loss through the FMM's
    # forward passes with the kernel's derivatives at the observers
    rr = (op.apply(s) - d).contiguous()
    go = op.observation_gradients(s, rr)["obs_locs"].cpu().numpy()
    ms_obs = _events_ms(torch, lambda: op.observation_gradients(s, rr), args.steps, stream)
    g = grad_step().cpu().numpy()
    r = Dop.apply(s_np) - d.cpu().numpy()
    gdd = ThreeD.direct_gradients(K, obs, on, sl, sn, sw, s_np, r)
    gd = gdd["x"]
    err = float(np.linalg.norm(g - gd) / np.linalg.norm(gd))
    err_obs = float(np.linalg.norm(go - gdd["obs_locs"]) / np.linalg.norm(gdd["obs_locs"]))
    y = op.apply(s_np)
    err_f = float(np.linalg.norm(y - Dop.apply(s_np)) / np.linalg.norm(Dop.apply(s_np)))
    print(json.dumps({
        "metric": METRIC, "value": len(obs) / (ms / 1e3), "unit": "points*RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded bumpy fault, free-surface observers)", "config": misfit_config(),
        "clocks": clk.summary(), "gpu_launches": 2 * op.last_launches() * args.steps,
        "forward_ms": ms_fwd, "vertex_gradient_ms": ms_vert,
        "vertex_gradient_direct_ms": ms_vert_direct, "observer_gradient_ms": ms_obs,
        "phases_ms_forward": phases,
        "rel_err_vs_direct": {"forward": err_f, "gradient_ds": err,
                              "gradient_vertices_fmm_vs_direct_pass": err_vert,
                              "gradient_observers_fmm_vs_direct_pass": err_obs}, "setup_s": setup_s,
        "setup_phases_s": setup_phases([op])}), flush=True)


def solve_config(n_subdiv, n_points):
    return {"workload": "exterior Laplace Dirichlet solve on a bumpy sphere r = 1 + 0.1 Y "
                        "(icosphere subdivided %d times, %d points), data of 10 interior unit "
                        "charges, second-kind combined-layer system (1/2 I - D + S) mu = g"
                        % (n_subdiv, n_points),
            "kernels": ["LaplaceSingle", "LaplaceDouble"], "n_points": n_points, "n_rhs": 1,
            "fmm": {"order_requested": ORDER, "surface_points": 295, "mac": MAC,
                    "min_pts_per_cell": LEAF, "d": D, "account_for_small_cells": False},
            "solver": "GMRES(50) to 1e-10: FP64 (FP64 compressed operators) and refined "
                      "(inner GMRES on the precision form, FP64 residuals)",
            "step": "one apply of the system with the precision-form operators (S and D)",
            "l2": "inputs larger than L2 at full size; no flush"}


def run_solve(args, rank, world, local):
    from tbempy import meshes
    v, t = meshes.bumpy_sphere(args.solve_subdiv)
    locs, nrm, w = meshes.points_from_mesh(v, t)
    N = len(locs)
    q = meshes.interior_charges()
    g = sum(1.0 / (4 * np.pi * np.linalg.norm(locs - p, axis=1)) for p in q)
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        oracle.build()
        frac = args.cpu_fraction
        ops = [oracle.OracleFMM(k, locs, nrm, locs, nrm, w, MAC, ORDER, LEAF, D)
               for k in ("LaplaceSingle", "LaplaceDouble")]
        ts = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            for o in ops:
                o.apply(g, list_fraction=frac)
            if i >= args.warmup:
                ts.append((time.perf_counter() - t0) / frac)
        tt = float(np.median(ts))
        value = N / tt
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "points*RHS/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded bumpy sphere)", "config": solve_config(args.solve_subdiv, N),
            "cpu_baseline": {"value": value, "unit": "points*RHS/s", "cores": oracle.max_threads(),
                             "kind": "port", "sample": "both oracle operators on the leading %.2g "
                                                       "of every task list, extrapolated" % frac},
            "e2e": {"value": value, "unit": "points*RHS/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    from tbempy import ThreeD, solve
    cfg = ThreeD.FMMConfig(MAC, ORDER, LEAF, D, False)
    kernels = (ThreeD.LaplaceSingle(), ThreeD.LaplaceDouble())
    t0 = time.perf_counter()
    ops = {p: [ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision=p, device=local)
               for K in kernels] for p in ("mixed", "fp64_compressed")}
    setup_s = time.perf_counter() - t0
    A32 = solve.exterior_dirichlet_system(ops["mixed"][0].apply, ops["mixed"][1].apply)
    A64 = solve.exterior_dirichlet_system(ops["fp64_compressed"][0].apply,
                                          ops["fp64_compressed"][1].apply)
    gt = torch.tensor(g, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        A32(gt)
        A64(gt)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = _events_ms(torch, lambda: A32(gt), args.steps, stream)
        ms64 = _events_ms(torch, lambda: A64(gt), 1, stream)
    # the FP64 solve and the refined solve, both to 1e-10
    counts = {"fp64": 0, "mixed": 0}

    def counted(A, key):
        def f(x):
            counts[key] += 1
            return A(x)
        return f

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x64, info, its64 = solve.gmres(counted(A64, "fp64"), gt, restart=50, tol=1e-10, maxiter=400)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    res64 = float(torch.linalg.norm(A64(x64) - gt) / torch.linalg.norm(gt))
    n64_plain = counts["fp64"]
    counts = {"fp64": 0, "mixed": 0}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xr, hist = solve.refined_solve(counted(A64, "fp64"), counted(A32, "mixed"), gt, tol=1e-10,
                                   inner_tol=1e-6)
    torch.cuda.synchronize()
    tref = time.perf_counter() - t0
    resr = float(torch.linalg.norm(A64(xr) - gt) / torch.linalg.norm(gt))
    # the field at 1,000 exterior points against the charges' potential
    rng = np.random.default_rng(8)
    d = rng.normal(size=(1000, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    X = d * rng.uniform(2.0, 3.0, 1000)[:, None]
    XN = np.tile([0.0, 0.0, 1.0], (1000, 1))
    mu = xr.cpu().numpy()
    u = (-ThreeD.DirectOperator(kernels[1], X, XN, locs, nrm, w).apply(mu)
         + ThreeD.DirectOperator(kernels[0], X, XN, locs, nrm, w).apply(mu))
    exact = sum(1.0 / (4 * np.pi * np.linalg.norm(X - p, axis=1)) for p in q)
    ext_err = float(np.linalg.norm(u - exact) / np.linalg.norm(exact))
    print(json.dumps({
        "metric": METRIC, "value": N / (ms / 1e3), "unit": "points*RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded bumpy sphere, interior charges)",
        "config": solve_config(args.solve_subdiv, N), "clocks": clk.summary(),
        "gpu_launches": sum(o.last_launches() for o in ops["mixed"]) * args.steps,
        "fp64_system_apply_ms": ms64,
        "fp64_solve": {"seconds": t64, "gmres_iterations": its64, "fp64_applies": n64_plain,
                       "relative_residual": res64, "converged": info == 0},
        "refined_solve": {"seconds": tref, "fp64_applies": counts["fp64"],
                          "precision_form_applies": counts["mixed"],
                          "history": [list(h) for h in hist], "relative_residual": resr},
        "solution_difference": float(torch.linalg.norm(xr - x64) / torch.linalg.norm(x64)),
        "exterior_rel_err_vs_analytic": ext_err, "setup_s": setup_s,
        "setup_phases_s": setup_phases(ops["mixed"] + ops["fp64_compressed"])}), flush=True)


def nearfield_config(n_subdiv, n_facets, shape, nnz):
    return {"workload": "nearfield matrix of the Laplace double layer on the unit icosphere "
                        "subdivided %d times (%d facets): GPU construction (sinh rule) and its CSR "
                        "apply (the nearfield correction's SpMV)" % (n_subdiv, n_facets),
            "kernel": "LaplaceDouble", "integrator": {"strategy": "sinh", "sinh_order": 5,
                                                      "obs_near_order": 2, "obs_far_order": 2,
                                                      "src_far_order": 2, "n_singular_steps": 8,
                                                      "far_threshold": 3.0},
            "csr": {"rows": shape[0], "cols": shape[1], "nnz": nnz, "index": "int64", "value": "f64"},
            "step": "one CSR apply, 1 RHS",
            "l2": "flushed before every timed step (256 MB write, outside the step timing)"}


def run_nearfield(args, rank, world, local):
    """The nearfield side of the operator: the GPU construction of the
    nearfield and farfield-correction matrices (timed once) and the CSR apply
    (SparseOperator::apply, cpp/sparse_operator.cpp:19-28), HBM-bound."""
    import torch
    torch.cuda.set_device(local)
    from tbempy import ThreeD, meshes
    v, f = meshes.icosphere(args.nf_subdiv)
    m = ThreeD.Mesh(v, f)
    K = ThreeD.LaplaceDouble()
    mthd = ThreeD.make_sinh_integrator(5, 2, 2, 2, 8, 3.0, K)
    t0 = time.perf_counter()
    near = ThreeD.nearfield_operator(m, m, mthd, m)
    t_near = time.perf_counter() - t0
    t0 = time.perf_counter()
    corr = ThreeD.farfield_correction_operator(m, m, mthd, m)
    t_corr = time.perf_counter() - t0
    rows, cols, nnz = near.n_rows(), near.n_cols(), near.nnz()
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, cols)
    xd = torch.tensor(x, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        near.apply(xd)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = _events_ms(torch, lambda: near.apply(xd), args.steps, stream, flush)
    # algorithmic bytes of one apply: values and column indices once, row
    # pointers, the output, and x once (a lower bound for the gathers)
    algo = nnz * (8 + 8) + (rows + 1) * 8 + rows * 8 + cols * 8
    hbm, _, peak_kind = peaks()
    achieved = algo / (ms / 1e3) / 1e9
    import scipy.sparse as sp
    A = sp.csr_matrix((near.values(), near.column_indices(), near.row_ptrs()), shape=(rows, cols))
    y_gpu = near.apply(x)
    err = float(np.linalg.norm(y_gpu - A @ x) / np.linalg.norm(A @ x))
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        A @ x
        ts.append(time.perf_counter() - t0)
    tc = float(np.median(ts))
    print(json.dumps({
        "metric": METRIC, "value": rows / (ms / 1e3), "unit": "nearfield rows*RHS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (icosphere)",
        "config": nearfield_config(args.nf_subdiv, m.n_facets(), (rows, cols), nnz),
        "clocks": clk.summary(), "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "kernel": "csr_kernel", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind + " copy bandwidth",
                     "traffic": None, "algorithmic_bytes_per_launch": algo},
        "construction_s": {"nearfield": t_near, "farfield_correction": t_corr,
                           "correction_nnz": corr.nnz()},
        "rel_err_vs_scipy": err,
        "cpu_baseline": {"value": rows / tc, "unit": "nearfield rows*RHS/s", "cores": 1, "kind": "port",
                         "sample": "scipy CSR matvec of the same matrix (a serial loop like "
                                   "SparseOperator::apply), median of 3"}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rhs", type=int, default=1)
    ap.add_argument("--cpu-fraction", type=float, default=0.01)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--grid", type=int, default=N_GRID,
                    help="quads per fault side (128 = the workload; smaller for ncu captures)")
    ap.add_argument("--kernels", default="both", choices=["both", "disp"])
    ap.add_argument("--m2l-path", type=int, default=0,
                    help="0 auto, 1 SIMT FP32, 2 tcgen05 M2L, 3 tcgen05 all, 4 compressed M2L")
    ap.add_argument("--m2l-rank-tol", type=float, default=1e-7,
                    help="singular-value cut of the compressed M2L")
    ap.add_argument("--workload", default="fault",
                    choices=["fault", "sphere", "batched", "misfit", "solve", "nearfield"],
                    help="fault: the elastic fault (default); sphere: plain FP64 Laplace single "
                         "layer on the 15,360-point icosphere; batched: Laplace double layer on "
                         "200 icospheres x 64 right-hand sides in one operator; misfit: the "
                         "gradient of the elastic misfit on the 64 x 64 bumpy fault")
    ap.add_argument("--meshes", type=int, default=200, help="batched workload: meshes")
    ap.add_argument("--batch-rhs", type=int, default=64, help="batched workload: right-hand sides")
    ap.add_argument("--nf-subdiv", type=int, default=6,
                    help="nearfield workload: icosphere subdivisions")
    ap.add_argument("--solve-subdiv", type=int, default=8,
                    help="solve workload: icosphere subdivisions (8: 3.9M points)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.workload != "fault":
        {"sphere": run_sphere, "batched": run_batched, "misfit": run_misfit,
         "solve": run_solve, "nearfield": run_nearfield}[args.workload](
            args, rank, world, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from tbempy import ThreeD
    locs, nrm, w, x = workload(args.grid)
    N = len(locs)
    cfg = ThreeD.FMMConfig(MAC, ORDER, LEAF, D, False)
    kernels = [ThreeD.ElasticDisplacement(MU, NU), ThreeD.ElasticTraction(MU, NU)]
    if args.kernels == "disp":
        kernels = kernels[:1]
    t0 = time.perf_counter()
    ops = [ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", device=local,
                              m2l_path=args.m2l_path, m2l_rank_tol=args.m2l_rank_tol)
           for K in kernels]
    setup_s = time.perf_counter() - t0
    # the evaluation kernels' denominators: FMA microbenchmark, before the timed region
    fma_peak = {"fp32": ThreeD.fma_peak_tflops(False, local), "fp64": ThreeD.fma_peak_tflops(True, local),
                "unit": "TFLOP/s", "method": "independent FMA chains on every SM, best of 3 ~10 ms runs"}
    n_rhs = args.rhs
    X = np.ascontiguousarray(np.tile(x, (n_rhs, 1)))
    xd = torch.tensor(X, device="cuda")
    yd = [torch.empty((n_rhs, op.n_rows()), dtype=torch.float64, device="cuda") for op in ops]
    stream = torch.cuda.current_stream()
    import ctypes as C
    sp = C.c_void_p(stream.cuda_stream if stream.cuda_stream else 1)
    # one step = every operator's apply, replayed as one CUDA graph with the
    # applies in parallel branches (tbem_fmm_graph_*): the two operators'
    # latency-bound passes overlap; the same kernels as the applies
    graph = ThreeD.FMMGraph(ops, [xd] * len(ops), yd, n_rhs=n_rhs)

    def step():
        graph.launch(sp)

    def step_sequential():
        for op in ops:
            op.apply(xd)

    for _ in range(args.warmup):
        step()
        step_sequential()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    torch.cuda.synchronize()

    def timed_region(fn):
        """Mean device ms of fn over args.steps runs, CUDA events on the
        stream; L2 flushed before every run (a 256 MB write, outside the
        events): the M2L operator planes alone would fit in L2."""
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        pairs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(args.steps)]
        for e0, e1 in pairs:
            flush.fill_(1)
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return sum(e0.elapsed_time(e1) for e0, e1 in pairs) / args.steps

    # -- device-resident timed region: the graph
    with ClockSampler(local) as clk:
        ms = timed_region(step)
        # the same step with the applies one after the other on one stream,
        # per-phase CUDA events recorded between the passes (read after it):
        # the phases and the M2L kernel's launch time of the roofline
        for op in ops:
            op.phase_times()  # drop the warm-up marks
            op.set_timing(True)
        ms_seq = timed_region(step_sequential)
    launches = sum(op.last_launches() for op in ops) * args.steps
    phase = {}       # ms per step (both operators)
    m2l_launch = []  # ms of the M2L kernel per launch, per operator
    for op in ops:
        for name, t in op.phase_times():
            phase[name] = phase.get(name, 0.0) + t
            if name == "m2l":
                m2l_launch.append(t)
        op.set_timing(False)
    value, sec = aggregate(ms / 1e3, len(ops) * N * n_rhs, dist, "cuda")
    ms = sec * 1e3

    # -- end to end through the public API with host buffers (pinned): the
    # slip copied to the device, the graph launched (tbem_fmm_graph_launch),
    # both results copied back, all inside the timed step
    xh = torch.tensor(X).pin_memory()
    yh = [torch.empty((n_rhs, op.n_rows()), dtype=torch.float64).pin_memory() for op in ops]

    def step_e2e():
        xd.copy_(xh, non_blocking=True)
        graph.launch(sp)
        for y, d in zip(yh, yd):
            y.copy_(d, non_blocking=True)
        torch.cuda.synchronize()

    for _ in range(2):
        step_e2e()
    if dist:
        dist.barrier()
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_e2e()  # ends with the device-to-host copies of the results
        e2e_s += time.perf_counter() - t0
    e2e_s /= args.steps
    e2e_value, e2e_s = aggregate(e2e_s, len(ops) * N * n_rhs, dist, "cuda")

    # -- accuracy against the FP64 direct sum on 4,096 random rows
    rng = np.random.default_rng(7)
    rows = np.sort(rng.choice(N, N_ERR_ROWS, replace=False))
    errs = {}
    for K, op, y in zip(kernels, ops, yh):
        direct = ThreeD.DirectOperator(K, locs[rows], nrm[rows], locs, nrm, w)
        exact = direct.apply(x)
        got = y[0].numpy().reshape(3, N)[:, rows].reshape(-1)
        errs[type(K).__name__] = float(np.linalg.norm(got - exact) / np.linalg.norm(exact))

    # -- roofline of the dominant kernel: the M2L products (one launch per
    # operator and apply), timed by the events of the timed region
    hbm, bf16, peak_kind = peaks()
    fl = [m2l_flops(op, n_rhs) for op in ops]
    launch_s = float(np.mean(m2l_launch)) / 1e3
    tensor = fl[0]["tensor"] is not None and all(op.tc_tile() > 0 for op in ops)
    per_launch = float(np.mean([f["tensor" if tensor else "reference"] for f in fl]))
    achieved = per_launch / launch_s / 1e12
    ref_form = float(np.mean([f["reference"] for f in fl]))
    traffic = None
    if tensor and args.grid == N_GRID and n_rhs == 1:
        traffic = M2L_TC_DRAM_BYTES

    # -- the plain FP64 form on the same workload
    plain = None
    if not args.no_plain:
        pops = [ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64", device=local)
                for K in kernels]
        for op in pops:
            op.apply(xd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for op in pops:
            op.apply(xd)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1)
        perr = {}
        for K, op in zip(kernels, pops):
            direct = ThreeD.DirectOperator(K, locs[rows], nrm[rows], locs, nrm, w)
            exact = direct.apply(x)
            got = op.apply(x).reshape(3, N)[:, rows].reshape(-1)
            perr[type(K).__name__] = float(np.linalg.norm(got - exact) / np.linalg.norm(exact))
        plain = {"ms_per_step": pms, "points_rhs_per_s": len(pops) * N * n_rhs / (pms / 1e3),
                 "rel_err_vs_direct": perr, "speedup_mixed_vs_plain": pms / ms}
        del pops

    cpu = None
    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        cops, _, cores = cpu_operators(locs, nrm, w, threads)
        calib = cpu_calibration(cops, x, args.cpu_fraction)
        t_full = cpu_apply_seconds(cops, x, args.cpu_fraction) * calib["ratio"]
        del cops
        cpu = {"value": 2 * N / t_full, "unit": "points*RHS/s", "cores": cores, "kind": "port",
               "sample": "oracle FMM apply of both kernels on the leading %.3g of every task "
                         "list, extrapolated to a full apply and scaled by the full / sampled "
                         "ratio of one full displacement apply (%.1f s)"
                         % (args.cpu_fraction, calib["full_apply_s"]),
               "calibration": calib}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points*RHS/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic (seeded dipping-fault mesh, tapered slip)",
            "config": config_dict(n_rhs),
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": "points*RHS/s",
                    "h2d_bytes_per_step": 8 * X.size,
                    "d2h_bytes_per_step": 8 * sum(y.numel() for y in yh)},
            "gpu_launches": launches,
            "ms_per_step_sequential": ms_seq,
            "roofline": {"bound": "tensor",
                         "kernel": ("tc_gemm_kernel: compressed M2L products, tcgen05 3xBF16"
                                    if tensor else "grouped_gemm_kernel: M2L products, FP32 SIMT"),
                         "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                         "frac": achieved / bf16,
                         "peak_kind": peak_kind + " bf16 dense (burst)",
                         "traffic": traffic,
                         "flops_per_launch": per_launch,
                         "launch_ms": launch_s * 1e3,
                         "reference_form_flops_per_launch": ref_form,
                         "reference_form_effective_tflops": ref_form / launch_s / 1e12},
            "phases_ms": phase,
            "rel_err_vs_direct": errs,
            "plain_fp64": plain,
            "fma_peak_measured": fma_peak,
            "cpu_baseline": cpu,
            "setup_s": setup_s,
            "setup_phases_s": setup_phases(ops),
            "m2l_ranks": [list(op.m2l_ranks()) for op in ops],
            "tc_tiles": [op.tc_tile() for op in ops],
            "p2p_threads_per_target": [op.p2p_block() for op in ops],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
