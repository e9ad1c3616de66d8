"""Benchmark of the FEM linear-solve path on one GB300 (or N replicas).

Workload (default): 96^3 Q1 scalar diffusion, a = exp(g) with g a squared-exponential Gaussian
random field (correlation 0.1, sigma 1.5), f ~ U[-1,1] per node, zero Dirichlet boundary by
projection: n = 912,673 dofs, 24,137,569 nonzeros.  A step is one solve from x = 0 to an FP64
relative residual ||b - A x|| / ||b|| <= 1e-8 (FP32 Jacobi-CG inner loop, FP64 iterative
refinement), inputs resident in HBM.  The matrix (204 MB of values + columns) is larger than the
129 MB L2, so no L2 flush is needed between steps.

Printed (rank 0, one JSON line): value = solve time (ms), e2e = the same solve through the public
API with host-resident inputs (matrix + rhs copied in, solution copied out, inside the timed
region), roofline of the dominant kernel (the BSR SpMV) against the measured HBM copy peak,
cpu_baseline = the oracle's FP64 Jacobi-PCG on the host cores (bounded sample).

``--impl reference`` times the reference's CPU implementation of this path (the oracle port of
Warp's CG; the reference's own CPU build needs its LLVM JIT, which is not available here) on all
host cores for the same workload, and prints the same line with impl=reference.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Solve time to 1e-8 rel. residual: learned-FCG vs Jacobi-CG; bsr_mv HBM GB/s"
WORKLOAD = ("96^3 Q1 lognormal diffusion (GRF l=0.1, sigma=1.5), 912,673 dofs, 24.1M nnz; "
            "Jacobi-CG FP32 inner + FP64 refinement to 1e-8 FP64 relative residual")


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, gpu_index: int = 0):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
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
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _barrier_max(value: float, ws: int):
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline_sample(system, gpu_iters: int, budget_s: float = 20.0):
    """Oracle FP64 Jacobi-PCG on all host threads, bounded: run up to ~budget_s of CPU work and
    scale the per-iteration time to the iteration count of a full solve."""
    import numpy as np

    import oracle

    A = system.A
    nnz = A.nnz_sync()
    off = A.offsets.cpu().numpy()
    cols = A.columns[:nnz].cpu().numpy()
    vals = A.values[:nnz].cpu().numpy()
    b = system.b.cpu().numpy()
    dinv = oracle.inverse_diagonal_f32(off, cols, vals)
    threads = oracle.max_threads()
    t0 = time.perf_counter()
    _, it_probe, _ = oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=20, nthreads=threads)
    probe = time.perf_counter() - t0
    per_iter = probe / max(it_probe, 1)
    n_iter = int(max(20, min(gpu_iters, budget_s / max(per_iter, 1e-6))))
    t0 = time.perf_counter()
    _, it_done, rel = oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=n_iter, nthreads=threads)
    dt = time.perf_counter() - t0
    full_iters = it_done if rel <= 1e-8 else max(gpu_iters, it_done)
    est_ms = dt / max(it_done, 1) * full_iters * 1e3
    return {"value": est_ms, "unit": "ms", "cores": threads, "kind": "port",
            "sample": f"{it_done} FP64 Jacobi-PCG iterations of the same 96^3 system in {dt:.2f} s on {threads} "
                      f"threads (rel. residual {rel:.2e}); scaled to {full_iters} iterations"}


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    import numpy as np
    import torch

    import oracle
    from warp_gb300 import problems

    system = problems.diffusion(args.res, sigma=1.5, corr_length=0.1, seed=args.seed)
    A = system.A
    nnz = A.nnz_sync()
    off = A.offsets.cpu().numpy()
    cols = A.columns[:nnz].cpu().numpy()
    vals = A.values[:nnz].cpu().numpy()
    b = system.b.cpu().numpy()
    dinv = oracle.inverse_diagonal_f32(off, cols, vals)
    threads = oracle.max_threads()
    # bounded sample per step: a fixed number of iterations; the full-solve time is scaled by the
    # iteration count the same oracle needs for 1e-8 (measured once, bounded by a wall budget)
    per_step_iters = args.ref_iters
    for _ in range(args.warmup):
        oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=5, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, it, rel = oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=per_step_iters,
                                    nthreads=threads)
        times.append((time.perf_counter() - t0) / max(it, 1))
    per_iter = statistics.median(times)
    full_iters = args.ref_full_iters
    value = per_iter * full_iters * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": "replicas"},
        "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": "port",
                         "sample": f"{per_step_iters} FP64 Jacobi-PCG iterations per step on {threads} threads, "
                                   f"median {per_iter * 1e3:.3f} ms/iteration, scaled to {full_iters} iterations"},
        "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """Kernel sequences for ncu (launch lists and single-kernel captures) on the bench workload."""
    import torch

    from warp_gb300 import problems, sparse
    from warp_gb300.optim import linear

    torch.cuda.set_device(0)
    system = problems.diffusion(args.res, sigma=1.5, corr_length=0.1, seed=args.seed)
    A = system.A
    torch.cuda.synchronize()
    torch.cuda.empty_cache()  # keep the device footprint of the capture small (assembly temporaries)
    if args.profile == "spmv":
        x = torch.randn(A.nrow, dtype=torch.float32, device="cuda")
        y = torch.empty_like(x)
        for _ in range(8):
            sparse.bsr_mv(A, x, y)
    elif args.profile == "cg":
        x = torch.zeros_like(system.b)
        linear.cg(A, system.b, x, tol=1e-12, atol=0.0, maxiter=30, M=linear.preconditioner(A, "diag"),
                  check_every=30, use_cuda_graph=False)
    else:
        solver = linear.RefinedSolver(A, M=linear.preconditioner(A, "diag"), inner_tol=args.inner_tol)
        solver.solve(system.b, tol=1e-8)
    torch.cuda.synchronize()
    print("profile run done", flush=True)
    return 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--res", type=int, nargs="+", default=[96, 96, 96])
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--inner-tol", type=float, default=1e-5)
    p.add_argument("--mv-launches", type=int, default=50)
    p.add_argument("--ref-iters", type=int, default=50)
    p.add_argument("--ref-full-iters", type=int, default=2000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--profile", choices=["spmv", "cg", "solve"], default=None,
                   help="run a fixed kernel sequence for an ncu capture and exit (prints no bench line): "
                        "spmv = 8 bsr_mv launches, cg = 30 eager (non-graph) Jacobi-CG iterations, "
                        "solve = one refined solve")
    args = p.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)

    import numpy as np
    import torch

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from warp_gb300 import problems, sparse
    from warp_gb300.optim import linear

    system = problems.diffusion(args.res, sigma=1.5, corr_length=0.1, seed=args.seed + rank)
    A = system.A
    n = A.nrow
    nnz = A.nnz_sync()
    M = linear.preconditioner(A, "diag")
    solver = linear.RefinedSolver(A, M=M, inner_tol=args.inner_tol)
    stream = torch.cuda.current_stream()

    # ---- warm-up -----------------------------------------------------------------------------
    for _ in range(args.warmup):
        x64, info = solver.solve(system.b, tol=1e-8)
    torch.cuda.synchronize()

    # ---- timed solves (inputs resident) ------------------------------------------------------
    infos = []
    sampler = ClockSampler(local)
    with sampler:
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = solver.kernel_launches
        e0.record(stream)
        for _ in range(args.steps):
            x64, info = solver.solve(system.b, tol=1e-8)
            infos.append(info)
        e1.record(stream)
        solver.kernel_launches_timed = solver.kernel_launches - launches0
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    ms = _barrier_max(ms, ws)
    clocks = sampler.summary()

    # ---- flexible CG with the multigrid preconditioner (set-up timed separately) -------------
    from warp_gb300 import multigrid

    torch.cuda.synchronize()
    s0 = time.perf_counter()
    mg = multigrid.MultigridPreconditioner(A, system.geo, system.coef)
    fsolver = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=args.inner_tol)
    torch.cuda.synchronize()
    mg_setup_ms = (time.perf_counter() - s0) * 1e3
    for _ in range(args.warmup):
        fsolver.solve(system.b, tol=1e-8)
    torch.cuda.synchronize()
    finfos = []
    with ClockSampler(local) as fsampler:
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            _, finfo = fsolver.solve(system.b, tol=1e-8)
            finfos.append(finfo)
        f1.record(stream)
        torch.cuda.synchronize()
    fcg_ms = _barrier_max(f0.elapsed_time(f1) / args.steps, ws)

    # ---- SpMV roofline (dominant kernel) -----------------------------------------------------
    hbm_peak, peak_kind = _peaks()
    x = torch.randn(n, dtype=torch.float32, device="cuda")
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    for _ in range(3):
        sparse.bsr_mv(A, x, y)
    torch.cuda.synchronize()
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m0.record(stream)
    for _ in range(args.mv_launches):
        sparse.bsr_mv(A, x, y)
    m1.record(stream)
    torch.cuda.synchronize()
    mv_s = m0.elapsed_time(m1) / args.mv_launches * 1e-3
    mv_bytes = nnz * (4 + 4) + (n + 1) * 4 + n * 4 + n * 4
    mv_gbs = mv_bytes / mv_s / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "bsr_mv_96cube.md")) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    traffic = float(line.split(":")[1])
    except OSError:
        pass

    # ---- end to end through the public API with host-resident inputs -------------------------
    off_h = A.offsets.cpu().pin_memory()
    col_h = A.columns[:nnz].cpu().pin_memory()
    val_h = A.values[:nnz].cpu().pin_memory()
    b_h = system.b.cpu().pin_memory()
    x_h = torch.empty(n, dtype=torch.float64).pin_memory()
    h2d = off_h.numel() * 4 + col_h.numel() * 4 + val_h.numel() * 4 + b_h.numel() * 4
    d2h = n * 8
    E = sparse.bsr_zeros(n, n, torch.float32)
    E.offsets = torch.empty_like(A.offsets)
    E.columns = torch.empty(nnz, dtype=torch.int32, device="cuda")
    E.values = torch.empty(nnz, dtype=torch.float32, device="cuda")
    E.nnz = nnz
    bE = torch.empty(n, dtype=torch.float32, device="cuda")
    E.offsets.copy_(off_h)
    E.columns.copy_(col_h)
    E.values.copy_(val_h)
    ME = linear.preconditioner(E, "diag")
    solverE = linear.RefinedSolver(E, M=ME, inner_tol=args.inner_tol)

    def e2e_step():
        # a user's repeated solve: new matrix values / rhs arrive from the host every step
        E.offsets.copy_(off_h, non_blocking=True)
        E.columns.copy_(col_h, non_blocking=True)
        E.values.copy_(val_h, non_blocking=True)
        bE.copy_(b_h, non_blocking=True)
        linear.refresh_preconditioner(ME, E)
        xs, inf = solverE.solve(bE, tol=1e-8)
        x_h.copy_(xs, non_blocking=True)
        return inf

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    g1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = _barrier_max(g0.elapsed_time(g1) / args.steps, ws)

    inner_iters = [i["inner_iterations"] for i in infos]
    outer = [i["outer"] for i in infos]
    # counted by the solver: residuals, argument stores, CG inits, solution updates, 3 per CG iteration
    gpu_launches = int(solver.kernel_launches_timed)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(system, int(statistics.median(inner_iters)))

    line = {
        "metric": METRIC,
        "value": ms,
        "unit": "ms",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "solver": "jacobi_cg_refined", "n_dofs": n, "nnz": nnz,
                   "parallelism": f"replicas{ws}", "l2": "inputs > L2 (matrix 204 MB vs 129 MB L2), no flush",
                   "inner_tol": args.inner_tol},
        "roofline": {"bound": "hbm", "kernel": "k_bsr_mv<1,1,float>", "achieved": mv_gbs, "peak": hbm_peak,
                     "unit": "GB/s", "frac": mv_gbs / hbm_peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": mv_bytes, "traffic": traffic, "launch_us": mv_s * 1e6},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "jacobi_cg_ms": ms,
        "mg_fcg_ms": fcg_ms,
        "mg_fcg_iterations": statistics.median([f["inner_iterations"] for f in finfos]),
        "mg_fcg_rel_residual": max(f["rel_residual"] for f in finfos),
        "mg_fcg_fallbacks": fsolver.fallbacks,
        "mg_setup_ms": mg_setup_ms,
        "mg_levels": mg.describe(),
        "bsr_mv_gbs": mv_gbs,
        "inner_iterations": statistics.median(inner_iters),
        "outer_iterations": statistics.median(outer),
        "rel_residual": max(i["rel_residual"] for i in infos),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
