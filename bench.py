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


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the host cores (the oracle
    port; the reference's own build needs its checkout, absent on the GPU machine)."""
    if rank != 0:
        return
    locs, nrm, w, x = workload()
    threads = os.cpu_count() or 1
    frac = args.cpu_fraction
    # built once, like the operator of the GPU arm; each step is one apply
    ops, setup, cores = cpu_operators(locs, nrm, w, threads)
    samples = []
    for i in range(args.warmup + args.steps):
        t_full = cpu_apply_seconds(ops, x, frac)
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
                                   "extrapolated to a full apply" % frac},
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
            "l2": "flushed before every timed step (256 MB write, outside the step timing)"}


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
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
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
    n_rhs = args.rhs
    X = np.ascontiguousarray(np.tile(x, (n_rhs, 1)))
    xd = torch.tensor(X, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        for op in ops:
            op.apply(xd)

    for _ in range(args.warmup):
        step()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2
    torch.cuda.synchronize()

    # -- device-resident timed region (per-phase CUDA events recorded on the
    # operators' stream inside it, read after it)
    for op in ops:
        op.phase_times()  # drop the warm-up marks
        op.set_timing(True)
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        # L2 flushed before every timed step (a 256 MB write, outside the
        # step's events): the M2L operator planes alone would fit in L2
        pairs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(args.steps)]
        for e0, e1 in pairs:
            flush.fill_(1)
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in pairs) / args.steps
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

    # -- end to end through the C ABI with host buffers (pinned)
    xh = torch.tensor(X).pin_memory()
    yh = [torch.empty((n_rhs, op.n_rows()), dtype=torch.float64).pin_memory() for op in ops]
    from tbempy import _lib
    L = _lib.lib()
    import ctypes as C

    def step_e2e():
        for op, y in zip(ops, yh):
            _lib.check(L.tbem_fmm_apply(op._h, C.c_void_p(xh.data_ptr()),
                                        C.c_void_p(y.data_ptr()), n_rhs, None))

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
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and tensor and args.grid == N_GRID and n_rhs == 1:
        # DRAM bytes of one launch of the tensor kernel on this workload, from a
        # one-pass ncu capture of this bench
        traffic = json.load(open(tpath)).get("m2l_tc_dram_bytes_per_launch")

    # -- the plain FP64 form on the same workload
    plain = None
    if not args.no_plain:
        pops = [ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64", device=local)
                for K in kernels]
        for op in pops:
            op.apply(xd)
        torch.cuda.synchronize()
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
        t_full = cpu_apply_seconds(cops, x, args.cpu_fraction)
        del cops
        cpu = {"value": 2 * N / t_full, "unit": "points*RHS/s", "cores": cores, "kind": "port",
               "sample": "oracle FMM apply of both kernels on the leading %.3g of every task "
                         "list, extrapolated to a full apply (%.1f s measured)"
                         % (args.cpu_fraction, t_full * args.cpu_fraction)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points*RHS/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic (seeded dipping-fault mesh, tapered slip)",
            "config": config_dict(n_rhs),
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": "points*RHS/s",
                    "h2d_bytes_per_step": 2 * 8 * X.size,
                    "d2h_bytes_per_step": 8 * sum(y.numel() for y in yh)},
            "gpu_launches": launches,
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
            "cpu_baseline": cpu,
            "setup_s": setup_s,
            "m2l_ranks": [list(op.m2l_ranks()) for op in ops],
            "tc_tiles": [op.tc_tile() for op in ops],
            "p2p_threads_per_target": [op.p2p_block() for op in ops],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
