"""Benchmark of the FEM linear-solve path on one GB300 (or N replicas).

Workload (default): 96^3 Q1 scalar diffusion, a = exp(g) with g a squared-exponential Gaussian
random field (correlation 0.1, sigma 1.5), f ~ U[-1,1] per node, zero Dirichlet boundary by
projection: n = 912,673 dofs, 24,137,569 nonzeros.  A step is one solve from x = 0 to an FP64
relative residual ||b - A x|| / ||b|| <= 1e-8 with the learned preconditioner: flexible CG in FP32
whose preconditioner is a multigrid V-cycle with the trained conv-net fine-level smoother (bf16
tcgen05 layers), inside FP64 iterative refinement; operator and preconditioner resident in HBM
(their set-up is timed separately).  The matrix (204 MB of values + columns) is larger than the
129 MB L2, so no L2 flush is needed between steps.  The same system is also solved by the plain
Jacobi-CG drop-in (the method the learned one is measured against) and by flexible CG with the Jacobi-smoothed
V-cycle (the method without the network).

Printed (rank 0, one JSON line): value = learned-FCG solve time (ms); e2e = the same solve through
the public API with the right-hand side copied in from pinned host memory and the FP64 solution
copied out inside the timed region (e2e_with_setup adds the matrix and coefficient copies and the
whole preconditioner set-up); roofline of the dominant kernel (the BSR SpMV) against the measured
HBM copy peak; cpu_baseline = the oracle's FP64 Jacobi-PCG on the host cores (bounded sample).

``--impl reference`` times the reference's CPU implementation of this path (the oracle port of
Warp's CG; the reference's own CPU build needs its LLVM JIT, which is not available here) on all
host cores for the same workload, and prints the same line with impl=reference.
"""

from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Solve time to 1e-8 rel. residual: learned-FCG vs Jacobi-CG; bsr_mv HBM GB/s"
# scalar type of the fine level's stencil coefficients inside the V-cycle (the flexible solver's own
# product and the FP64 refinement keep fp32 values); resolved to a torch dtype where torch is imported
VCYCLE_FINE = "bf16"
WORKLOAD = ("96^3 Q1 lognormal diffusion (GRF l=0.1, sigma=1.5), 912,673 dofs, 24.1M nnz; "
            "learned-preconditioned FCG (multigrid V-cycle + trained conv-net smoother) FP32 inner + FP64 "
            "refinement to 1e-8 FP64 relative residual")


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _fine_values():
    import torch

    return torch.bfloat16 if VCYCLE_FINE == "bf16" else torch.float32


def _tensor_peak():
    """Dense bf16 tensor peak (TFLOP/s) for a kernel timed alone: the measured burst figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured (burst)"
    except Exception:
        return 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling around the timed region.

    The sampler is started before the warm-up (so that spawning nvidia-smi does not stall the host
    inside the timed region) and polls every 50 ms; each sample carries nvidia-smi's timestamp, and
    summary() keeps the samples whose timestamps fall inside the window set by mark()."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.proc = None
        # raw samples: GB_CLOCKS_DIR if set, else the system temporary directory (the summary goes into
        # the bench line either way)
        self.path = os.path.join(os.environ.get("GB_CLOCKS_DIR") or tempfile.gettempdir(), f"clocks_{os.getpid()}.csv")
        self.gpu = gpu_index
        self.window = None

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
            # nvidia-smi's start-up (driver attach, first query) must not overlap the timed region: wait
            # for its first sample (at most 5 s)
            t_end = time.time() + 5.0
            while time.time() < t_end and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def mark(self, t0, t1):
        """The timed region, as host datetimes."""
        self.window = (t0, t1)

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
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                    rows.append((ts, float(parts[2]), float(parts[3]),
                                 {nm for nm, v in zip(names, parts[6:10]) if v.lower().startswith("active")}))
                except ValueError:
                    continue
        except OSError:
            pass
        inside = rows
        if self.window is not None and rows:
            t0, t1 = self.window
            pad = datetime.timedelta(milliseconds=60)
            inside = [r for r in rows if t0 - pad <= r[0] <= t1 + pad]
            if not inside:  # region shorter than the sampling interval: the nearest sample
                mid = t0 + (t1 - t0) / 2
                inside = [min(rows, key=lambda r: abs((r[0] - mid).total_seconds()))]
        sm = [r[1] for r in inside]
        reasons = set().union(*[r[3] for r in inside]) if inside else set()
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(r[2] for r in inside) if inside else None,
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


def _event_ms(fn, reps: int, warmup: int = 1) -> float:
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def bench_batched(args, hbm_peak):
    """4096 uneven 2-D Q1 diffusion systems (n ~ U{16..128} cells per side, GRF l=0.1, sigma=1), one
    persistent batched Jacobi-CG launch (autotuned, CUDA graph) to 1e-6 relative residual each."""
    import numpy as np
    import torch

    from warp_gb300 import batched
    from warp_gb300.optim import linear

    rng = np.random.default_rng(args.seed)
    ncells_all = rng.integers(16, 129, size=args.batch_count)
    ws, rank = _dist()
    # N GPUs: the systems are split by batched.shard (weak in work per GPU, no collective)
    mine = batched.shard((ncells_all + 1) ** 2, rank, ws)
    ncells = ncells_all[mine]
    t0 = time.perf_counter()
    Am, b, offs = batched.q1_batch_2d(ncells, sigma=1.0, corr_length=0.1, seed=args.seed)
    build_s = time.perf_counter() - t0
    M = linear.preconditioner(Am, "diag")
    solver = batched.BatchedCG(Am, offs, M._inv_diag, 1e-6, 0.0, 0, config="auto")
    x = torch.zeros_like(b)
    t0 = time.perf_counter()
    solver.solve(b, x)  # autotunes on the first call
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t0

    def step():
        x.zero_()
        solver.solve(b, x)

    ms = _barrier_max(_event_ms(step, args.steps, warmup=2), ws)
    it = solver.iters.cpu().numpy()
    rows = np.diff(offs.cpu().numpy())
    nnz_rows = (3 * ncells + 1) ** 2
    # algorithmic bytes: per subproblem iteration the matrix (8 B / nonzero + 4 B / row offsets) and
    # 48 B / row of vector traffic (Ap write; p, x, r, Ap, dinv read, x, r write; r, dinv, p read, p write)
    algo = float((it * (nnz_rows * 8 + rows * 52)).sum())
    gbs = algo / (ms * 1e-3) / 1e9
    conv = float((solver.rr <= solver.atol_sq).float().mean())
    return {"workload": f"{args.batch_count} Q1 2-D diffusion systems, n ~ U{{16..128}} cells/side, "
                        f"{int(rows.sum())} rows, {int(nnz_rows.sum())} nnz on this rank, Jacobi-CG to 1e-6 each",
            "ms": ms, "systems_per_s": args.batch_count / (ms * 1e-3), "launches_per_solve": 2,
            "sharding": f"{len(mine)} of {args.batch_count} systems on rank {rank} of {ws} (batched.shard)",
            "config": {k: v for k, v in solver.config.items() if k != "tuned_ms"},
            "iterations": {"min": int(it.min()), "median": float(np.median(it)), "max": int(it.max())},
            "converged_fraction": conv, "status": int(solver.status.item()),
            "algorithmic_bytes": algo, "achieved_gbs": gbs, "frac_of_hbm": gbs / hbm_peak,
            "build_s": build_s, "autotune_s": tune_s}


def bench_assembly(args, system, hbm_peak):
    """96^3 bilinear assembly through fem.integrate: the default direct compact-BSR assembly, and the
    triplet (bsr_set_from_triplets) and row-compress constructions."""
    import numpy as np
    import torch

    from warp_gb300 import fem

    geo = system.geo
    space = fem.make_polynomial_space(geo, degree=1)
    coef = torch.from_numpy(np.asarray(system.coef, np.float32)).cuda()  # resident: not part of assembly
    fields = {"u": fem.make_trial(space), "v": fem.make_test(space)}

    def assemble(construction):
        def run():
            m = fem.integrate(fem.diffusion_form, fields=fields, values={"nu": coef},
                              bsr_options={"construction": construction})
            m.nnz_sync()
        return run

    ms = _event_ms(assemble("auto"), 5, warmup=2)
    tri_ms = _event_ms(assemble("triplets"), 3)
    rc_ms = _event_ms(assemble("row_compress"), 3)
    A = system.A
    T = geo.cell_count() * 64
    nnz = A.nnz_sync()
    # triplet construction: read T triplets (row, col, value), write the BSR (the sort passes are
    # implementation cost, reported separately)
    algo = T * (8 + 4) + nnz * (4 + 4) + (A.nrow + 1) * 4
    # direct assembly: read the cell coefficients, write offsets (count pass + scan) and the BSR
    direct = geo.cell_count() * 4 + nnz * (4 + 4) + 2 * (A.nrow + 1) * 4
    sort_passes = 5
    return {"ms": ms, "construction": "direct compact-BSR assembly (fem.integrate default)", "nnz": nnz,
            "algorithmic_bytes": direct, "achieved_gbs": direct / (ms * 1e-3) / 1e9,
            "frac_of_hbm": direct / (ms * 1e-3) / 1e9 / hbm_peak,
            "triplets": T, "triplets_ms": tri_ms, "triplets_algorithmic_bytes": algo,
            "triplets_frac_of_hbm": algo / (tri_ms * 1e-3) / 1e9 / hbm_peak,
            "triplets_sort_bytes": sort_passes * 12 * T,
            "row_compress_ms": rc_ms, "row_compress_frac_of_hbm": algo / (rc_ms * 1e-3) / 1e9 / hbm_peak,
            "note": "coefficients resident on the device; every variant returns the same matrix bit for bit; the "
                    "triplet construction writes 56.6 M triplets and radix-sorts them (sort passes x 12 B x T "
                    "reported separately)"}


def _oracle_residual_3x3(A, b, x):
    """||b - A x|| / ||b|| in FP64 on the host (oracle BSR product of the fp32 3x3 blocks)."""
    import numpy as np

    import oracle

    nnz = A.nnz_sync()
    r = b.cpu().numpy().astype(np.float64) - oracle.bsr_mv_f64(
        A.offsets.cpu().numpy(), A.columns[:nnz].cpu().numpy(), A.values[:nnz].cpu().numpy().reshape(-1),
        x.cpu().numpy().astype(np.float64), block_shape=(3, 3))
    return float(np.linalg.norm(r) / np.linalg.norm(b.cpu().numpy().astype(np.float64)))


def bench_elasticity(args, hbm_peak):
    """64^3 Q1 vec3 elasticity (E lognormal sigma=1 i.i.d., nu=0.3, gravity, x=0 clamped): 3x3 bsr_mv
    bandwidth and the refined Jacobi-CG solve to 1e-8."""
    import torch

    from warp_gb300 import problems, sparse
    from warp_gb300.optim import linear

    s = problems.elasticity((args.elasticity_res,) * 3, sigma=1.0, seed=args.seed)
    A = s.A
    nnz = A.nnz_sync()
    n = A.nrow * 3
    xv = torch.randn(n, device="cuda")
    yv = torch.empty_like(xv)
    mv_ms = _event_ms(lambda: sparse.bsr_mv(A, xv, yv), 20, warmup=3)
    mv_bytes = nnz * (36 + 4) + (A.nrow + 1) * 4 + 2 * n * 4
    solver = linear.RefinedSolver(A, M=linear.preconditioner(A, "diag"), inner_tol=args.inner_tol)
    solver.solve(s.b, tol=1e-8)
    infos, xs = [], []

    def step():
        x_, info_ = solver.solve(s.b, tol=1e-8)
        infos.append(info_)
        xs.append(x_)

    ms = _event_ms(step, 2, warmup=0)
    # bf16 storage of the matrix values for the FP32 inner loop (the FP64 residual keeps fp32 values)
    bsolver = linear.RefinedSolver(A, M=linear.preconditioner(A, "diag"), inner_tol=args.inner_tol,
                                   inner_values=A.values[:nnz].to(torch.bfloat16).contiguous())
    binfos = []
    bsolver.solve(s.b, tol=1e-8)
    bms = _event_ms(lambda: binfos.append(bsolver.solve(s.b, tol=1e-8)[1]), 2, warmup=0)
    return {"workload": f"{args.elasticity_res}^3 Q1 vec3 elasticity, {A.nrow} block rows, {nnz} blocks",
            "jacobi_cg_refined_bf16_values_ms": bms, "bf16_inner_iterations": binfos[-1]["inner_iterations"],
            "bf16_outer_iterations": binfos[-1]["outer"], "bf16_rel_residual": binfos[-1]["rel_residual"],
            "bsr_mv_us": mv_ms * 1e3, "bsr_mv_gbs": mv_bytes / (mv_ms * 1e-3) / 1e9,
            "bsr_mv_frac_of_hbm": mv_bytes / (mv_ms * 1e-3) / 1e9 / hbm_peak,
            "jacobi_cg_refined_ms": ms, "inner_iterations": infos[-1]["inner_iterations"],
            "rel_residual": infos[-1]["rel_residual"], "oracle_rel_residual": _oracle_residual_3x3(A, s.b, xs[-1])}


def bench_elasticity_large(args, hbm_peak):
    """128^3 Q1 vec3 elasticity (E lognormal sigma=1.5, GRF correlation length 0.05, nu=0.3, gravity,
    x=0 clamped; 2.15 M nodes, 6.4 M dofs): assembly (triplet and row-compress constructions), 3x3
    bsr_mv with fp32 and bf16 values, and the refined flexible-CG solve to 1e-8 with the vec3 multigrid
    V-cycle (fp32 and bf16 inner values)."""
    import numpy as np
    import torch

    from warp_gb300 import fem, multigrid, problems, sparse
    from warp_gb300.optim import linear

    res = args.elasticity_large_res
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = problems.elasticity((res,) * 3, sigma=1.5, corr_length=0.05, seed=args.seed)
    torch.cuda.synchronize()
    problem_s = time.perf_counter() - t0
    A = s.A
    nnz = A.nnz_sync()
    n = A.nrow * 3
    ncells = res ** 3
    # assembly alone (fem.integrate of the bilinear form), both constructions
    lam, mu = fem.q1.lame_from_young(s.coef, 0.3)
    lam_t = torch.from_numpy(lam.astype(np.float32)).cuda()
    mu_t = torch.from_numpy(mu.astype(np.float32)).cuda()
    space = fem.make_polynomial_space(s.geo, degree=1, dtype="vec3")
    fields = {"u": fem.make_trial(space), "v": fem.make_test(space)}
    asm = {}
    for construction in ("auto", "triplets", "row_compress"):
        def assemble():
            M_ = fem.integrate(fem.linear_elasticity_form, fields=fields, values={"lame": (lam_t, mu_t)},
                               bsr_options={"construction": construction})
            M_.nnz_sync()
        asm[construction] = _event_ms(assemble, 2, warmup=1)
        torch.cuda.empty_cache()
    triplets = ncells * 64
    asm_bytes = triplets * (8 + 36) + nnz * (4 + 36) + (A.nrow + 1) * 4
    direct_bytes = ncells * 8 + nnz * (4 + 36) + 2 * (A.nrow + 1) * 4
    # 3x3 SpMV, fp32 and bf16 values
    xv = torch.randn(n, device="cuda")
    yv = torch.empty_like(xv)
    mv_ms = _event_ms(lambda: sparse.bsr_mv(A, xv, yv), 10, warmup=3)
    mv_bytes = nnz * (36 + 4) + (A.nrow + 1) * 4 + 2 * n * 4
    Ab = sparse.BsrMatrix(A.nrow, A.ncol, A.block_shape, torch.bfloat16)
    Ab.offsets, Ab.columns, Ab.nnz = A.offsets, A.columns, A.nnz
    Ab.values = A.values[:nnz].to(torch.bfloat16).contiguous()
    mvb_ms = _event_ms(lambda: sparse.bsr_mv(Ab, xv, yv), 10, warmup=3)
    mvb_bytes = nnz * (18 + 4) + (A.nrow + 1) * 4 + 2 * n * 4
    # multigrid set-up and the refined flexible-CG solves
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mg = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=("x-",))
    torch.cuda.synchronize()
    mg_setup_s = time.perf_counter() - t0
    out = {"workload": f"{res}^3 Q1 vec3 elasticity, {A.nrow} block rows ({n} dofs), {nnz} blocks, E lognormal "
                       f"sigma 1.5 GRF l=0.05",
           "problem_build_s": problem_s,
           "assembly_ms": asm["auto"], "assembly_direct_bytes": direct_bytes,
           "assembly_frac_of_hbm": direct_bytes / (asm["auto"] * 1e-3) / 1e9 / hbm_peak,
           "assembly_triplets_ms": asm["triplets"], "assembly_row_compress_ms": asm["row_compress"],
           "assembly_triplets_algorithmic_bytes": asm_bytes,
           "assembly_triplets_frac_of_hbm": asm_bytes / (asm["triplets"] * 1e-3) / 1e9 / hbm_peak,
           "bsr_mv_us": mv_ms * 1e3, "bsr_mv_gbs": mv_bytes / (mv_ms * 1e-3) / 1e9,
           "bsr_mv_frac_of_hbm": mv_bytes / (mv_ms * 1e-3) / 1e9 / hbm_peak,
           "bsr_mv_bf16_us": mvb_ms * 1e3, "bsr_mv_bf16_gbs": mvb_bytes / (mvb_ms * 1e-3) / 1e9,
           "bsr_mv_bf16_frac_of_hbm": mvb_bytes / (mvb_ms * 1e-3) / 1e9 / hbm_peak,
           "mg_levels": mg.describe(), "mg_setup_ms": mg_setup_s * 1e3,
           "mg_omega": [round(lv.omega, 4) for lv in mg.levels]}
    solver = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=args.inner_tol, inner_maxiter=5000)
    solver.solve(s.b, tol=1e-8, max_outer=10)
    infos, xs = [], []

    def solve_once():
        x_, info_ = solver.solve(s.b, tol=1e-8, max_outer=10)
        infos.append(info_)
        xs.append(x_)

    ms = _event_ms(solve_once, 2, warmup=0)
    out["mg_fcg_fp32_ms"] = ms
    out["mg_fcg_fp32_oracle_rel_residual"] = _oracle_residual_3x3(A, s.b, xs[-1])
    out["mg_fcg_fp32_inner_iterations"] = infos[-1]["inner_iterations"]
    out["mg_fcg_fp32_outer_iterations"] = infos[-1]["outer"]
    out["mg_fcg_fp32_rel_residual"] = infos[-1]["rel_residual"]
    out["mg_fcg_fp32_converged"] = infos[-1]["converged"]
    out["mg_fcg_fp32_fallbacks"] = solver.fallbacks
    # bf16 matrix values inside the V-cycle (fine level), fp32 values in the flexible solver's product
    del mg, solver
    torch.cuda.empty_cache()
    mg16 = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=("x-",), fine_values=torch.bfloat16)
    solver16 = linear.RefinedSolver(A, M=mg16, method="fcg", inner_tol=args.inner_tol, inner_maxiter=5000)
    solver16.solve(s.b, tol=1e-8, max_outer=10)
    infos16, xs16 = [], []

    def solve16():
        x_, info_ = solver16.solve(s.b, tol=1e-8, max_outer=10)
        infos16.append(info_)
        xs16.append(x_)

    out["mg_fcg_bf16_vcycle_ms"] = _event_ms(solve16, 2, warmup=0)
    out["mg_fcg_bf16_vcycle_inner_iterations"] = infos16[-1]["inner_iterations"]
    out["mg_fcg_bf16_vcycle_converged"] = infos16[-1]["converged"]
    out["mg_fcg_bf16_vcycle_oracle_rel_residual"] = _oracle_residual_3x3(A, s.b, xs16[-1])
    # the 3-channel learned smoother (vec3 network, trained on elasticity fields with the 128^3 statistics)
    from warp_gb300 import learned

    if os.path.exists(learned.ELASTICITY_WEIGHTS):
        del mg16, solver16
        torch.cuda.empty_cache()
        net3 = learned.ConvNet.load(learned.ELASTICITY_WEIGHTS)
        mgL = multigrid.MultigridPreconditioner(A, s.geo, s.coef, faces=("x-",), fine_values=torch.bfloat16)
        mgL.smoother = learned.LearnedSmoother(net3, mgL, s.coef)
        solverL = linear.RefinedSolver(A, M=mgL, method="fcg", inner_tol=args.inner_tol, inner_maxiter=5000)
        solverL.solve(s.b, tol=1e-8, max_outer=10)
        infosL, xsL = [], []

        def solveL():
            x_, info_ = solverL.solve(s.b, tol=1e-8, max_outer=10)
            infosL.append(info_)
            xsL.append(x_)

        out["learned_fcg_ms"] = _event_ms(solveL, 2, warmup=0)
        out["learned_fcg_inner_iterations"] = infosL[-1]["inner_iterations"]
        out["learned_fcg_converged"] = infosL[-1]["converged"]
        out["learned_fcg_fallbacks"] = solverL.fallbacks
        out["learned_fcg_oracle_rel_residual"] = _oracle_residual_3x3(A, s.b, xsL[-1])
        out["learned_weights"] = os.path.relpath(learned.ELASTICITY_WEIGHTS, ROOT)
    out["note"] = ("flexible CG with the vec3 geometric V-cycle (point-Jacobi smoothing, damping 4/(3 rho) per "
                   "level); fp32 values, and bf16 fine-level values inside the V-cycle with fp32 values in the "
                   "flexible solver's product (bf16 values as the refinement's inner operator diverge on this "
                   "field, sigma 1.5); learned_fcg: the same bf16 cycle with the 3-channel conv-net smoother "
                   "(16 hidden channels, tcgen05 layers) on the fine level")
    return out


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    import numpy as np

    import oracle
    from oracle import fem_q1

    # the system is built on the host by the oracle (FP64 stencil assembly, Dirichlet projection):
    # the same workload as the GPU arm's, without the product library
    off, cols, vals, b = fem_q1.diffusion_system_3d(tuple(args.res), sigma=1.5, corr_length=0.1, seed=args.seed)
    dinv = oracle.inverse_diagonal_f32(off, cols, vals)
    threads = oracle.max_threads()
    # each step is one complete FP64 Jacobi-PCG solve to 1e-8 relative residual (about 0.5 s on 16
    # threads at 96^3); --ref-max-iters bounds it
    for _ in range(args.warmup):
        oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=5, nthreads=threads)
    times, iters, rels = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, it, rel = oracle.pcg_f64(off, cols, vals, b, inv_diag=dinv, tol=1e-8, maxiter=args.ref_max_iters,
                                    nthreads=threads)
        times.append(time.perf_counter() - t0)
        iters.append(it)
        rels.append(rel)
    value = statistics.median(times) * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": "replicas",
                   "input": "system built on the host by the oracle (FP64 stencil assembly + Dirichlet projection, "
                            "oracle/fem_q1.py); the product library is not loaded"},
        "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": "port",
                         "sample": f"one full FP64 Jacobi-PCG solve of the same 96^3 system per step on {threads} "
                                   f"threads ({iters[-1]} iterations, rel. residual {rels[-1]:.2e})"},
        "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """Kernel sequences for ncu (launch lists and single-kernel captures) on the bench workload."""
    import numpy as np
    import torch

    from warp_gb300 import problems, sparse
    from warp_gb300.optim import linear

    torch.cuda.set_device(0)
    if args.profile == "conv":  # 3 launches of one hidden tcgen05 layer on the 97^3 node grid
        import warp_gb300._native as N
        from warp_gb300 import learned

        dims = tuple(r + 1 for r in args.res)
        src = learned.to_planar(torch.randn(int(np.prod(dims)), 16, device="cuda"), dims)
        dst = torch.zeros_like(src)
        Wt = (torch.randn(27, 16, 16, device="cuda") * 0.1).to(torch.bfloat16).contiguous()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        for _ in range(3):
            N.check(N.lib().gb_conv3_fwd_tc(*dims, 0, src.data_ptr(), Wt.data_ptr(), dst.data_ptr(), None, None, None,
                                            None, 0.0, st.data_ptr(), torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        print("profile run done", flush=True)
        return 0
    if args.profile == "convnet":  # 3 applications of the learned smoother (features + one network launch)
        from warp_gb300 import learned, multigrid

        system = problems.diffusion(tuple(args.res), sigma=1.5, corr_length=0.1, seed=0)
        mg = multigrid.MultigridPreconditioner(system.A, system.geo, system.coef)
        sm = learned.LearnedSmoother(learned.ConvNet.load(learned.DEFAULT_WEIGHTS), mg, system.coef)
        r = torch.randn(system.A.nrow, device="cuda") * (1 - mg.levels[0].mask)
        w = torch.empty_like(r)
        for _ in range(3):
            sm.launch(torch.cuda.current_stream().cuda_stream, r.data_ptr(), w.data_ptr())
        torch.cuda.synchronize()
        assert int(mg.status.item()) == 0
        print("profile run done", flush=True)
        return 0
    if args.profile == "vcycle":  # 3 eager V-cycles (stencil-form levels) on the 97^3 node grid
        from warp_gb300 import multigrid, problems

        system = problems.diffusion(args.res, sigma=1.5, corr_length=0.1, seed=args.seed)
        mg = multigrid.MultigridPreconditioner(system.A, system.geo, system.coef)
        r = torch.randn(system.A.nrow, device="cuda") * (1 - mg.levels[0].mask)
        for _ in range(3):
            mg.apply(r)
        torch.cuda.synchronize()
        assert int(mg.status.item()) == 0
        print("profile run done", flush=True)
        return 0
    if args.profile == "batched":  # 512 uneven systems, two eager batched launches (fixed shape)
        from warp_gb300 import batched

        rng = np.random.default_rng(args.seed)
        Am, b, offs = batched.q1_batch_2d(rng.integers(16, 129, size=512), seed=args.seed)
        Mb = linear.preconditioner(Am, "diag")
        bs = batched.BatchedCG(Am, offs, Mb._inv_diag, 1e-6, 0.0, 0, use_cuda_graph=False,
                               config={"threads": 256, "lanes_per_row": 2, "small_rows": 0})
        x = torch.zeros_like(b)
        for _ in range(2):
            x.zero_()
            bs.solve(b, x)
        torch.cuda.synchronize()
        assert int(bs.status.item()) == 0
        print("profile run done", flush=True)
        return 0
    system = problems.diffusion(args.res, sigma=1.5, corr_length=0.1, seed=args.seed)
    A = system.A
    torch.cuda.synchronize()
    torch.cuda.empty_cache()  # keep the device footprint of the capture small (assembly temporaries)
    if args.profile == "assembly":  # fem.integrate once by each construction (direct, triplets, row compress)
        from warp_gb300 import fem

        space = fem.make_polynomial_space(system.geo, degree=1)
        coef = torch.from_numpy(np.asarray(system.coef, np.float32)).cuda()
        fields = {"u": fem.make_trial(space), "v": fem.make_test(space)}
        for construction in ("auto", "triplets", "row_compress"):
            m = fem.integrate(fem.diffusion_form, fields=fields, values={"nu": coef},
                              bsr_options={"construction": construction})
            m.nnz_sync()
            del m
            torch.cuda.empty_cache()
        torch.cuda.synchronize()
        print("profile run done", flush=True)
        return 0
    if args.profile == "spmv":
        x = torch.randn(A.nrow, dtype=torch.float32, device="cuda")
        y = torch.empty_like(x)
        for _ in range(8):
            sparse.bsr_mv(A, x, y)
    elif args.profile == "cg":
        x = torch.zeros_like(system.b)
        linear.cg(A, system.b, x, tol=1e-12, atol=0.0, maxiter=30, M=linear.preconditioner(A, "diag"),
                  check_every=30, use_cuda_graph=False)
    elif args.profile == "jacobi_solve":
        solver = linear.RefinedSolver(A, M=linear.preconditioner(A, "diag"), inner_tol=args.inner_tol)
        solver.solve(system.b, tol=1e-8)
    else:  # the learned-FCG solve of the bench line (set-up, one warm-up solve, one solve)
        from warp_gb300 import learned, multigrid

        net = learned.ConvNet.load(args.weights)
        mg = multigrid.MultigridPreconditioner(A, system.geo, system.coef, fine_values=_fine_values(),
                                               omega=net.cycle_omega or "auto")
        mg.smoother = learned.LearnedSmoother(net, mg, system.coef, backend="tc")
        # eager launches (host check per iteration) so that every kernel of the solve is listed
        solver = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=args.inner_tol, use_cuda_graph=False)
        for _ in range(2):
            solver.solve(system.b, tol=1e-8)
    torch.cuda.synchronize()
    print("profile run done", flush=True)
    return 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--res", type=int, nargs="+", default=[96, 96, 96])
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--inner-tol", type=float, default=None,
                   help="inner tolerance of every refined solve (default: the solver's own, 1e-4 for the "
                        "flexible solves and 1e-5 for the Krylov drop-ins)")
    p.add_argument("--mv-launches", type=int, default=50)
    p.add_argument("--ref-max-iters", type=int, default=5000,
                   help="iteration bound of the reference arm's FP64 Jacobi-PCG solve")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the batched, assembly and elasticity (64^3 and 128^3) measurements")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--elasticity-res", type=int, default=64)
    p.add_argument("--elasticity-large-res", type=int, default=128,
                   help="cells per axis of the large elasticity extra (0 skips it)")
    p.add_argument("--weights", default=os.path.join(ROOT, "warp_gb300", "data", "smoother_q1_diffusion.npz"))
    p.add_argument("--profile", choices=["spmv", "cg", "jacobi_solve", "solve", "conv", "convnet", "batched", "vcycle",
                                         "assembly"],
                   default=None,
                   help="run a fixed kernel sequence for an ncu capture and exit (prints no bench line): "
                        "spmv = 8 bsr_mv launches, cg = 30 eager (non-graph) Jacobi-CG iterations, "
                        "jacobi_solve = one refined Jacobi-CG solve, solve = two learned-FCG solves (eager launches), "
                        "conv = 3 launches of one tcgen05 conv layer on the node grid, convnet = 3 applications of "
                        "the learned smoother (features kernel + whole-network launch), batched = two launches of "
                        "the batched CG on 512 uneven systems, vcycle = 3 eager multigrid V-cycles (stencil levels), "
                        "assembly = one 96^3 fem.integrate per construction (direct, triplets, row compress)")
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
    stream = torch.cuda.current_stream()
    from warp_gb300 import learned, multigrid

    def timed(solver, b, steps, sample_clocks=False):
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.__enter__()
        for _ in range(args.warmup):
            solver.solve(b, tol=1e-8)
        torch.cuda.synchronize()
        infos = []
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = solver.kernel_launches
        w0 = datetime.datetime.now()
        e0.record(stream)
        xlast = None
        for _ in range(steps):
            xlast, info = solver.solve(b, tol=1e-8)
            infos.append(info)
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.mark(w0, datetime.datetime.now())
        launches = solver.kernel_launches - launches0
        if ws > 1:
            torch.distributed.barrier()
        if sampler:
            sampler.__exit__(None, None, None)
        ms_ = _barrier_max(e0.elapsed_time(e1) / steps, ws)
        solver.last_x = xlast.cpu().numpy()  # outside the timed region: checked against the oracle below
        return ms_, infos, launches, (sampler.summary() if sampler else None)

    # ---- learned preconditioner: set-up (timed separately) and the headline solve -------------
    # the set-up is built twice and the second build timed: the first carries one-time costs (first
    # launches of the set-up kernels, allocator growth) that are not part of a solve's set-up
    for attempt in range(2):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        net = learned.ConvNet.load(args.weights)
        # the hierarchy in the damping the network was trained with (no per-level estimate to discard)
        lmg = multigrid.MultigridPreconditioner(A, system.geo, system.coef, fine_values=_fine_values(),
                                                omega=net.cycle_omega or "auto")
        lmg.smoother = learned.LearnedSmoother(net, lmg, system.coef, backend="tc")
        lsolver = linear.RefinedSolver(A, M=lmg, method="fcg", inner_tol=args.inner_tol)
        torch.cuda.synchronize()
        setup_ms = (time.perf_counter() - s0) * 1e3
    ms, linfos, llaunch, clocks = timed(lsolver, system.b, args.steps, sample_clocks=True)

    # ---- plain Jacobi-CG drop-in (the reference method for the speed-up) ----------------------
    M = linear.preconditioner(A, "diag")
    jsolver = linear.RefinedSolver(A, M=M, inner_tol=args.inner_tol)
    jms, jinfos, _, jclocks = timed(jsolver, system.b, args.steps, sample_clocks=True)
    # the same solve with three kernels per CG iteration under a conditional graph node (the
    # persistent cooperative launch switched off), for comparison
    jsolver3 = linear.RefinedSolver(A, M=M, inner_tol=args.inner_tol, persistent=False)
    j3ms, j3infos, _, _ = timed(jsolver3, system.b, max(3, args.steps // 4))

    # ---- the same flexible CG without the network (Jacobi-smoothed V-cycle) -------------------
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    mg = multigrid.MultigridPreconditioner(A, system.geo, system.coef, fine_values=_fine_values())
    fsolver = linear.RefinedSolver(A, M=mg, method="fcg", inner_tol=args.inner_tol)
    torch.cuda.synchronize()
    mg_setup_ms = (time.perf_counter() - s0) * 1e3
    fcg_ms, finfos, _, _ = timed(fsolver, system.b, args.steps)

    # ---- the learned solve with fp32 fine-level coefficients in the V-cycle, for comparison -----
    l32 = multigrid.MultigridPreconditioner(A, system.geo, system.coef, omega=net.cycle_omega or "auto")
    l32.smoother = learned.LearnedSmoother(net, l32, system.coef, backend="tc")
    l32solver = linear.RefinedSolver(A, M=l32, method="fcg", inner_tol=args.inner_tol)
    l32ms, l32infos, _, _ = timed(l32solver, system.b, max(3, args.steps // 4))
    del l32solver, l32
    # ... and with the flexible solver's product on the CSR matrix instead of the fine level's stencil form
    lcsr = linear.RefinedSolver(A, M=lmg, method="fcg", inner_tol=args.inner_tol, stencil_product=False)
    lcsr_ms, lcsr_infos, _, _ = timed(lcsr, system.b, max(3, args.steps // 4))
    del lcsr

    # ---- the learned smoother's layers (tensor-core roofline) ----------------------------------
    sm = lmg.smoother
    r_t = torch.randn(n, device="cuda") * (1 - lmg.levels[0].mask)
    w_t = torch.empty_like(r_t)
    for _ in range(3):
        sm.launch(stream.cuda_stream, r_t.data_ptr(), w_t.data_ptr())
    torch.cuda.synchronize()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(20):
        sm.launch(stream.cuda_stream, r_t.data_ptr(), w_t.data_ptr())
    c1.record(stream)
    torch.cuda.synchronize()
    smoother_us = c0.elapsed_time(c1) / 20 * 1e3
    net_flop = 2.0 * 27 * (16 * 16 * 3 + 16 * 1) * n  # useful MACs x 2 of the four layers
    net_tflops = net_flop / (smoother_us * 1e-6) / 1e12

    # ---- SpMV roofline (dominant kernel) -----------------------------------------------------
    hbm_peak, peak_kind = _peaks()
    x = torch.randn(n, dtype=torch.float32, device="cuda")
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    # mv_launches back-to-back launches captured in a CUDA graph (as the solvers run them; no host gaps
    # between launches), replayed after warm-up; the graph's events bracket exactly those launches
    mv_graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for _ in range(3):
            sparse.bsr_mv(A, x, y)
        with torch.cuda.graph(mv_graph, stream=side):
            for _ in range(args.mv_launches):
                sparse.bsr_mv(A, x, y)
    stream.wait_stream(side)
    for _ in range(2):
        mv_graph.replay()
    torch.cuda.synchronize()
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m0.record(stream)
    mv_graph.replay()
    m1.record(stream)
    torch.cuda.synchronize()
    mv_s = m0.elapsed_time(m1) / args.mv_launches * 1e-3
    del mv_graph
    mv_bytes = nnz * (4 + 4) + (n + 1) * 4 + n * 4 + n * 4
    mv_gbs = mv_bytes / mv_s / 1e9
    # fused Jacobi-PCG iteration: the SpMV (beta = 0) and 48 B of vector traffic per row
    jit_bytes = mv_bytes + 48 * n
    # the same number of bytes moved by a plain device copy (read + write = mv_bytes): the bandwidth a
    # single launch of this size reaches (ramp-up and tail included), for context beside the peak
    cbuf = torch.empty(mv_bytes // 8, dtype=torch.float32, device="cuda")
    cdst = torch.empty_like(cbuf)
    copy_s = _event_ms(lambda: cdst.copy_(cbuf), args.mv_launches, warmup=3) * 1e-3
    copy_gbs = mv_bytes / copy_s / 1e9
    del cbuf, cdst
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "bsr_mv_96cube.md")) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    traffic = float(line.split(":")[1])
    except OSError:
        pass

    # ---- end to end through the public API with host-resident inputs -------------------------
    b_h = system.b.cpu().pin_memory()
    x_h = torch.empty(n, dtype=torch.float64).pin_memory()
    bE = torch.empty(n, dtype=torch.float32, device="cuda")

    def e2e_step():
        # a user's solve: the right-hand side arrives from the host, the solution goes back
        bE.copy_(b_h, non_blocking=True)
        xs, inf = lsolver.solve(bE, tol=1e-8)
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
    h2d, d2h = n * 4, n * 8

    # with set-up: matrix, coefficient field and rhs from the host, preconditioner rebuilt, solve
    off_h = A.offsets.cpu().pin_memory()
    col_h = A.columns[:nnz].cpu().pin_memory()
    val_h = A.values[:nnz].cpu().pin_memory()
    coef_h = torch.from_numpy(np.asarray(system.coef, np.float32).reshape(-1)).pin_memory()
    E = sparse.bsr_zeros(n, n, torch.float32)
    E.offsets = torch.empty_like(A.offsets)
    E.columns = torch.empty(nnz, dtype=torch.int32, device="cuda")
    E.values = torch.empty(nnz, dtype=torch.float32, device="cuda")
    E.nnz = nnz
    coefE = torch.empty(coef_h.numel(), dtype=torch.float32, device="cuda")

    def e2e_setup_step():
        E.offsets.copy_(off_h, non_blocking=True)
        E.columns.copy_(col_h, non_blocking=True)
        E.values.copy_(val_h, non_blocking=True)
        coefE.copy_(coef_h, non_blocking=True)
        bE.copy_(b_h, non_blocking=True)
        pm = multigrid.MultigridPreconditioner(E, system.geo, coefE)
        pm.smoother = learned.LearnedSmoother(net, pm, coefE, backend="tc")
        sol = linear.RefinedSolver(E, M=pm, method="fcg", inner_tol=args.inner_tol)
        xs, inf = sol.solve(bE, tol=1e-8)
        x_h.copy_(xs, non_blocking=True)
        torch.cuda.synchronize()
        return inf

    e2e_setup_step()
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 3))):
        e2e_setup_step()
    e2e_setup_ms = (time.perf_counter() - t0) * 1e3 / max(1, min(args.steps, 3))
    h2d_setup = off_h.numel() * 4 + col_h.numel() * 4 + val_h.numel() * 4 + coef_h.numel() * 4 + n * 4

    # ---- one hidden tcgen05 conv layer alone (tensor-core roofline of the smoother's kernel) ------
    import warp_gb300._native as N

    dims = lmg.levels[0].dims
    csrc = sm.buf[0]
    cdst = torch.zeros_like(csrc)
    cst = torch.zeros(1, dtype=torch.int32, device="cuda")

    def conv_layer():
        N.check(N.lib().gb_conv3_fwd_tc(*dims, 0, csrc.data_ptr(), sm.Wt[1].data_ptr(), cdst.data_ptr(), None, None,
                                        None, None, 0.0, cst.data_ptr(), stream.cuda_stream), "conv layer")

    conv_ms = _event_ms(conv_layer, 20, warmup=3)
    conv_flop = 2.0 * 27 * 16 * 16 * n  # useful MACs x 2 of one 16 -> 16 layer over the node grid
    conv_tflops = conv_flop / (conv_ms * 1e-3) / 1e12
    tensor_peak, tensor_peak_kind = _tensor_peak()
    assert int(cst.item()) == 0
    del cdst

    # ---- FP64 oracle checks of the solutions (outside every timed region) -----------------------
    import oracle

    off_np = A.offsets.cpu().numpy()
    col_np = A.columns[:nnz].cpu().numpy()
    val_np = A.values[:nnz].cpu().numpy()
    b_np = system.b.cpu().numpy().astype(np.float64)
    threads = oracle.max_threads()
    t0 = time.perf_counter()
    x_ref, ref_it, ref_rel = oracle.pcg_f64(off_np, col_np, val_np, b_np.astype(np.float32),
                                            inv_diag=oracle.inverse_diagonal_f32(off_np, col_np, val_np), tol=1e-12,
                                            maxiter=20000, nthreads=threads)
    ref_s = time.perf_counter() - t0

    def oracle_check(xs):
        r = b_np - oracle.bsr_mv_f64(off_np, col_np, val_np, xs)
        return {"oracle_rel_residual": float(np.linalg.norm(r) / np.linalg.norm(b_np)),
                "oracle_rel_error": float(np.linalg.norm(xs - x_ref) / np.linalg.norm(x_ref))}

    oracle_solve = {"method": "oracle FP64 Jacobi-PCG (oracle.pcg_f64) on the same fp32 matrix", "tol": 1e-12,
                    "iterations": ref_it, "rel_residual": ref_rel, "seconds": ref_s, "threads": threads}

    inner_iters = [i["inner_iterations"] for i in linfos]
    outer = [i["outer"] for i in linfos]
    # counted by the solver: residuals, argument stores, FCG inits, solution updates, and per FCG
    # iteration its 4 kernels + the V-cycle's (learned smoother included)
    gpu_launches = int(llaunch)

    extras = {}
    if not args.no_extras:
        extras["assembly_96cube"] = bench_assembly(args, system, hbm_peak)
        extras["batched_uneven"] = bench_batched(args, hbm_peak)
        extras["elasticity"] = bench_elasticity(args, hbm_peak)
        if args.elasticity_large_res > 0:
            extras["elasticity_large"] = bench_elasticity_large(args, hbm_peak)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(system, int(statistics.median([i["inner_iterations"] for i in jinfos])))

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
        "dtype": "f32+f64 (bf16 conv net)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "solver": "learned_fcg_refined", "n_dofs": n, "nnz": nnz,
                   "parallelism": f"replicas{ws}", "l2": "inputs > L2 (matrix 204 MB vs 129 MB L2), no flush",
                   "inner_tol": lsolver.inner_tol, "jacobi_cg_inner_tol": jsolver.inner_tol,
                   "weights": os.path.relpath(args.weights, ROOT),
                   "mg_levels": lmg.describe(), "vcycle_fine_values": VCYCLE_FINE,
                   "fcg_product": "27-point stencil form of A (fp32)" if lsolver.inner.stencil_product else "CSR",
                   "jacobi_cg": "persistent cooperative launch" if jsolver.inner.persistent_active else "three kernels"},
        "roofline": {"bound": "hbm", "kernel": "k_bsr_mv<1,1,float>", "achieved": mv_gbs, "peak": hbm_peak,
                     "unit": "GB/s", "frac": mv_gbs / hbm_peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": mv_bytes, "traffic": traffic, "launch_us": mv_s * 1e6,
                     "timing": f"CUDA events around a CUDA-graph replay of {args.mv_launches} launches",
                     "same_size_copy_gbs": copy_gbs, "frac_of_same_size_copy": mv_gbs / copy_gbs},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "e2e_with_setup": {"value": e2e_setup_ms, "unit": "ms", "h2d_bytes_per_step": h2d_setup,
                           "d2h_bytes_per_step": d2h, "timing": "host wall clock, synchronised"},
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "roofline_conv": {"bound": "tensor", "kernel": "k_conv3_tc<0, false> (one 16->16 hidden layer, 97^3 nodes)",
                          "achieved": conv_tflops, "peak": tensor_peak, "unit": "TFLOP/s",
                          "frac": conv_tflops / tensor_peak, "peak_kind": tensor_peak_kind,
                          "algorithmic_flop": conv_flop, "launch_us": conv_ms * 1e3,
                          "timing": "CUDA events on the launching stream around 20 launches after 3 warm-up"},
        "oracle_solve": oracle_solve,
        "learned_fcg": {"ms": ms, "inner_iterations": statistics.median(inner_iters),
                        "outer_iterations": statistics.median(outer),
                        "rel_residual": max(i["rel_residual"] for i in linfos), "fallbacks": lsolver.fallbacks,
                        "setup_ms": setup_ms, "speedup_vs_jacobi_cg": jms / ms, "vcycle_fine_values": VCYCLE_FINE,
                        "fp32_vcycle_ms": l32ms, "stencil_product": lsolver.inner.stencil_product,
                        "csr_product_ms": lcsr_ms,
                        "fp32_vcycle_inner_iterations": statistics.median([i["inner_iterations"] for i in l32infos]),
                        **oracle_check(lsolver.last_x)},
        "jacobi_cg": {"ms": jms, "inner_iterations": statistics.median([i["inner_iterations"] for i in jinfos]),
                      "outer_iterations": statistics.median([i["outer"] for i in jinfos]),
                      "rel_residual": max(i["rel_residual"] for i in jinfos), "clocks": jclocks,
                      "iteration_frac_of_hbm": (jit_bytes * statistics.median([i["inner_iterations"] for i in jinfos])
                                                / (jms * 1e-3) / 1e9 / hbm_peak),
                      "iteration_bytes": jit_bytes, "persistent_launch": jsolver.inner.persistent_active,
                      "three_kernel_iteration": {
                          "ms": j3ms, "inner_iterations": statistics.median([i["inner_iterations"] for i in j3infos]),
                          "iteration_frac_of_hbm": (jit_bytes * statistics.median([i["inner_iterations"] for i in j3infos])
                                                    / (j3ms * 1e-3) / 1e9 / hbm_peak)},
                      **oracle_check(jsolver.last_x)},
        "mg_fcg_no_net": {"ms": fcg_ms, "inner_iterations": statistics.median([f["inner_iterations"] for f in finfos]),
                          "rel_residual": max(f["rel_residual"] for f in finfos), "fallbacks": fsolver.fallbacks,
                          "setup_ms": mg_setup_ms, "vcycle_fine_values": VCYCLE_FINE, **oracle_check(fsolver.last_x)},
        "conv_net": {"smoother_us": smoother_us, "launches": sm.kernels_per_apply, "useful_tflops": net_tflops,
                     "backend": "tcgen05 kind::f16 bf16 x bf16 -> fp32"},
        "bsr_mv_gbs": mv_gbs,
        **extras,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
