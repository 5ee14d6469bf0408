#!/usr/bin/env python
"""Benchmark of the sparse-solver hot path on one GB300.

Workload (the headline metric "MG-PCG time-to-1e-8 at 192^3, mixed vs FP64"):
-div(k grad u) on a 192^3 grid (7,077,888 unknowns, 49,324,032 nonzeros), k = exp(g)
with g a unit Gaussian field of correlation length 8 cells (seed 2), b ~ U[-1,1].
Multigrid-preconditioned CG: 5 levels, trilinear interpolation, R = P^T, Galerkin
RAP, Jacobi (omega 0.8) 2+2 sweeps, dense FP64 Cholesky on the 12^3 coarse level.
Stop at ||r||_2 <= 1e-8 ||b||_2, checked in FP64.

  * value: wall time of the mixed-precision solve (FP64 flexible CG outer iteration,
    BF16-stored FP32 V-cycle), hierarchy already built, CUDA events on the library's
    stream; lower is better.  The plain FP64 form is timed the same way (fp64_ms).
  * roofline: the FP64 form's dominant kernel (CG's product fused with (p, Ap)) timed alone
    with CUDA events, against HBM (two byte models) and against the FP64 pipe.
  * e2e: the same solve through the public C ABI with host buffers: per step b is
    copied from pinned host memory, the solve runs, x is copied back (operator and
    hierarchy resident, as the reference's set-up is untimed too).  cold_path adds the
    operator/transfer upload and the hierarchy set-up.
  * cpu_baseline: the CPU oracle (a restatement of the reference's algorithms) on all
    host cores: one complete FP64 solve of the same problem (hierarchy built untimed).

  * other_workloads: 256^2 CG + Jacobi, 128^3 FP64 MG-PCG (Chebyshev), the 1024^2 obstacle
    QP (MPRGP, multicolour PGS) and the 128^3 differentiable solve (--no-extra skips them).

Other modes print their own line and are not the headline: --amg, --mmg, --qp (solvers beside the
path), --spmv-only, --cg-jacobi, --transfers (profiling cases), --setup (the cold path in parts).

--impl reference times only that CPU implementation (rank 0; other ranks exit).
Multi-GPU: the path is not sharded here (one GPU per box); N ranks run N replicas.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID = 192
LEVELS = 5
RTOL = 1e-8
METRIC = "MG-PCG time-to-1e-8 at 192^3 (mixed BF16/FP32 V-cycle in FP64 FCG)"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self):
        return time.perf_counter()

    def keep(self, windows):
        self.windows = windows

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        wins = getattr(self, "windows", None)
        for t, l in self.lines:
            if wins and not any(a <= t <= b for a, b in wins):
                continue
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_problem(n_grid):
    from utopia_gb300 import problems as P

    return P.lognormal_mg(n_grid, LEVELS, seed=2)


def oracle_setup(A, Ps):
    import oracle as O

    O.build()
    Am = O.Matrix(A)
    t0 = time.perf_counter()
    mg = O.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
    return O, Am, mg, time.perf_counter() - t0


def oracle_solve(O, Am, mg, b, with_x=False):
    """One complete FP64 MG-PCG solve on the CPU oracle (hierarchy already built)."""
    nb = float(np.linalg.norm(b))
    t0 = time.perf_counter()
    x, st = O.cg_solve(Am, b, precond="mg", mg=mg, atol=RTOL * nb)
    dt = time.perf_counter() - t0
    return (dt, st, x) if with_x else (dt, st)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    A, Ps, b = make_problem(args.size)
    O, Am, mg, setup_s = oracle_setup(A, Ps)
    times = []
    for k in range(args.warmup + args.steps):
        dt, st = oracle_solve(O, Am, mg, b)
        if k >= args.warmup:
            times.append(dt)
    ms = float(np.mean(times)) * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"lognormal diffusion {args.size}^3, FP64 MG-PCG (5 levels, Jacobi 0.8 2+2, "
                               "Galerkin RAP, dense Cholesky coarse) on the CPU oracle", "grid": args.size,
                   "timed": "solve phase per step (hierarchy built before the timed region)"},
        "iterations": st["iterates"] + 1,
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": O.max_threads(), "kind": "port",
                         "sample": f"complete FP64 solves to ||r|| <= 1e-8 ||b|| ({st['iterates'] + 1} "
                                   f"iterations); hierarchy set-up {setup_s:.1f} s untimed"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_spmv_only(args):
    """The kernels of the roofline and of the V-cycle's fine sweeps, launched in a fixed order:
    FP64 y = A x (x2), FP32 y = A x (x2), BF16 y = A x (x2), BF16 Jacobi sweep (x2), on the
    lognormal operator."""
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    A, _, _ = P.lognormal_diffusion_3d(args.size, 2)
    ctx = U.Context(0)
    M = U.SparseMatrix(ctx, A)
    M32, M16 = M.cast(U.F32), M.cast(U.BF16)
    rng = np.random.default_rng(0)
    x64 = U.Vector(ctx, rng.standard_normal(A.nrows))
    y64 = U.Vector(ctx, n=A.nrows)
    x32 = U.Vector(ctx, rng.standard_normal(A.nrows), dtype=U.F32)
    b32 = U.Vector(ctx, rng.standard_normal(A.nrows), dtype=U.F32)
    y32 = U.Vector(ctx, n=A.nrows, dtype=U.F32)
    for _ in range(2):
        M.apply(x64, y64)
    for _ in range(2):
        M32.apply(x32, y32)
    for _ in range(2):
        M16.apply(x32, y32)
    for _ in range(2):
        M16.jacobi_sweep(b32, x32, 0.8, y32)
    ctx.synchronize()
    print(json.dumps({"spmv_only": True, "n": A.nrows, "nnz": A.nnz}))


def run_cg_jacobi(args):
    """Profiling case: FP64 CG with the Jacobi preconditioner on the lognormal operator, four
    iterations, every kernel launched individually (FP64 SpMV + (p, Ap), the CG vector kernels)."""
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    A = P.lognormal_diffusion_3d(args.size, 2)[0]
    ctx = U.Context(0)
    M = U.SparseMatrix(ctx, A)
    b = U.Vector(ctx, np.random.default_rng(0).uniform(-1, 1, A.nrows))
    x = U.Vector(ctx, n=A.nrows)
    cg = U.ConjugateGradient(ctx, atol=0.0, max_it=4, use_graphs=0)
    cg.set_preconditioner(U.InvDiagPreconditioner(ctx))
    cg.solve(M, b, x)
    ctx.synchronize()
    print(json.dumps({"cg_jacobi": True, "n": A.nrows, "iterations": cg.solution_status()["iterates"]}))


def run_amg(args):
    """AMG-PCG (algebraic multigrid with greedy agglomeration, coarsened to <= 4096 rows) on the
    lognormal operator: set-up and graph-timed solve, FP64 and mixed (BF16 levels, flexible CG),
    and the oracle's FP64 AMG-PCG on the host cores beside it.  One JSON line."""
    import torch
    import utopia_gb300 as U

    A, _, b = make_problem(args.size)
    n = A.nrows
    nb = float(np.linalg.norm(b))
    ctx = U.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    Am, bv, x = U.SparseMatrix(ctx, A), U.Vector(ctx, b), U.Vector(ctx, n=n)
    out = {"metric": f"AMG-PCG time-to-{RTOL} at {args.size}^3", "unit": "ms", "higher_is_better": False,
           "config": {"workload": f"lognormal diffusion {args.size}^3 (n={n}, nnz={A.nnz}), AlgebraicMultigrid "
                                  "(Agglomerate bmax 3, weight 1/3) to <= 4096 rows, Jacobi(0.8) 2+2, dense "
                                  "Cholesky coarse", "tolerance": f"||r|| <= {RTOL} ||b||"}}
    for name, prec in (("fp64", U.F64), ("mixed", U.BF16)):
        amg = U.AlgebraicMultigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                                   n_levels=0, max_coarse_rows=4096, precision=prec)
        cg = U.ConjugateGradient(ctx, atol=RTOL * nb, flexible=0 if prec == U.F64 else 1, max_it=2000)
        cg.set_preconditioner(amg)
        t0 = time.perf_counter()
        cg.update(Am)
        ctx.synchronize()
        setup = time.perf_counter() - t0
        times = []
        for i in range(args.warmup + args.steps):
            x.set(0.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            cg.apply(bv, x)
            e.record(stream)
            e.synchronize()
            if i >= args.warmup:
                times.append(s.elapsed_time(e))
        st = cg.solution_status()
        res = float(np.linalg.norm(b - A.matvec(x.numpy())) / nb)
        out[name] = {"ms": float(np.mean(times)), "setup_ms": setup * 1e3, "iterations": st["iterates"] + 1,
                     "rel_residual_fp64": res, "levels": amg.n_levels()}
    if not args.no_cpu:
        import oracle as O

        O.build()
        Ao = O.Matrix(A)
        t0 = time.perf_counter()
        Ps, _ = O.amg_hierarchy(Ao, n_levels=0, max_coarse_rows=4096)
        mg = O.Multigrid(Ao, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
        setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, st = O.cg_solve(Ao, b, precond="mg", mg=mg, atol=RTOL * nb, max_it=2000)
        out["cpu_baseline"] = {"value": (time.perf_counter() - t0) * 1e3, "unit": "ms", "kind": "port",
                               "cores": O.max_threads(), "iterations": st["iterates"] + 1,
                               "setup_ms": setup * 1e3, "sample": "one complete FP64 AMG-PCG solve on the oracle"}
    out["value"] = out["mixed"]["ms"]
    print(json.dumps(out), flush=True)


def run_transfers(args):
    """The transfers between the fine level and the next (trilinear P and R = P^T of the size^3 grid),
    BF16 values with FP32 vectors and FP64: restriction R x and prolongation y = P x + v, each timed
    by CUDA events around single launches with L2 flushed before each.  One JSON line."""
    import torch
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    ctx = U.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    Pm = U.SparseMatrix(ctx, P.interpolation_3d(args.size))
    Rm = Pm.transpose()
    P16, R16 = Pm.cast(U.BF16), Rm.cast(U.BF16)
    nf, nc = Pm.nrows, Pm.ncols
    rng = np.random.default_rng(0)
    rf32, xc32 = U.Vector(ctx, rng.standard_normal(nf), dtype=U.F32), U.Vector(ctx, rng.standard_normal(nc), dtype=U.F32)
    yc32, yf32 = U.Vector(ctx, n=nc, dtype=U.F32), U.Vector(ctx, n=nf, dtype=U.F32)
    rf64, yc64 = U.Vector(ctx, rng.standard_normal(nf)), U.Vector(ctx, n=nc)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def t(fn, reps=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            tot += s.elapsed_time(e)
        return tot / reps * 1e3

    out = {"metric": f"transfer times {args.size}^3 <-> {args.size // 2}^3", "unit": "us",
           "restrict_bf16_us": t(lambda: R16.apply(rf32, yc32)),
           "prolong_add_bf16_us": t(lambda: P16.apply_add(xc32, rf32, yf32)),
           "restrict_f64_us": t(lambda: Rm.apply(rf64, yc64)),
           "R_sell": R16.sell_info(), "P_sell": P16.sell_info(), "l2": "flushed (256 MB write) before each launch"}
    print(json.dumps(out), flush=True)


def run_setup(args):
    """The cold path of the headline solve in parts: operator upload (CSR from host arrays, validation,
    sliced-ELL layout), transfer uploads, transfer set-up (transposes), hierarchy set-up (Galerkin
    products, storage casts and layouts, coarse factorisation), the first solve (graph capture) and a
    second one.  Host-timed with a synchronisation around each part, three repetitions.  One JSON line."""
    import utopia_gb300 as U

    A, Ps, b = make_problem(args.size)
    ctx = U.Context(0)
    nb = float(np.linalg.norm(b))
    reps = []
    for _ in range(3):
        log = {}

        def part(tag, fn):
            ctx.synchronize()
            t0 = time.perf_counter()
            r = fn()
            ctx.synchronize()
            log[tag] = (time.perf_counter() - t0) * 1e3
            return r

        A_d = part("operator_upload_ms", lambda: U.SparseMatrix(ctx, A))
        P_d = part("transfer_upload_ms", lambda: [U.SparseMatrix(ctx, p) for p in Ps])
        b_d = part("rhs_upload_ms", lambda: U.Vector(ctx, b))
        mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                         precision=U.BF16)
        part("transfer_setup_ms", lambda: mg.set_transfer_operators(P_d))
        cg = U.ConjugateGradient(ctx, atol=RTOL * nb, flexible=1)
        cg.set_preconditioner(mg)
        x_d = U.Vector(ctx, n=A.nrows)
        part("hierarchy_setup_ms", lambda: cg.update(A_d))
        part("first_solve_ms", lambda: cg.apply(b_d, x_d))
        x_d.set(0.0)
        part("second_solve_ms", lambda: cg.apply(b_d, x_d))
        part("download_ms", lambda: x_d.numpy())
        reps.append(log)
        del cg, mg, A_d, P_d, b_d, x_d
    print(json.dumps({"metric": f"cold path in parts, {args.size}^3 mixed MG-PCG", "unit": "ms",
                      "repetitions": reps}), flush=True)


def qp_measure(ctx, N, scale, steps, eager=False, max_it=400000, pgs=True, pgs_max_it=None):
    """MPRGP and multicolour projected Gauss-Seidel on the N^2 obstacle problem (5-point
    Laplacian, Gaussian-bump lower bound, seed 3) with b = -1 (scale None, the problem as
    specified) or b = -scale h^2.  Complete solves timed by CUDA events on the library's
    stream (operator, bounds and b resident); stop at the projected-gradient norm 1e-8
    (MPRGP's own criterion; PGS stops on it too, evaluated every iteration)."""
    import torch
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-1.0 if scale is None else -scale * h * h)
    atol = 1e-8 if scale is None else 1e-8 * h * h
    stream = torch.cuda.ExternalStream(ctx.stream)
    Am, bv, x = U.SparseMatrix(ctx, A), U.Vector(ctx, b), U.Vector(ctx, n=A.nrows)
    lbv, ubv = U.Vector(ctx, lb), U.Vector(ctx, ub)
    out = {"n": A.nrows, "b": "-1" if scale is None else f"-{scale:g} h^2", "atol": atol}
    makers = {"mprgp": lambda: U.MPRGP(ctx, atol=atol, rtol=1e-30, max_it=max_it, use_graphs=0 if eager else 1)}
    if pgs:
        makers["pgs_multicolour"] = lambda: U.ProjectedGaussSeidel(
            ctx, atol=atol, max_it=pgs_max_it or max_it, projected_gradient_stop=1, use_graphs=0 if eager else 1)
    for name, make in makers.items():
        s = make()
        s.set_box_constraints(lbv, ubv)
        s.update(Am)
        times = []
        for i in range(1 + max(1, steps)):
            x.set(0.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = ctx.launch_count()
            e0.record(stream)
            s.apply(bv, x)
            e1.record(stream)
            e1.synchronize()
            if i >= 1:
                times.append(e0.elapsed_time(e1))
            launches = ctx.launch_count() - l0
        st = s.solution_status()
        xg = x.numpy()
        rec = {"ms": float(np.median(times)), "iterations": int(st["iterates"]), "converged": bool(st["converged"]),
               "active_fraction": float((xg == lb).mean()), "gpu_launches": int(launches)}
        rec["us_per_iteration"] = rec["ms"] * 1e3 / max(rec["iterations"], 1)
        out[name] = rec
    return out


def extra_workloads(ctx, args, stream):
    """The other workloads of the path, measured on the same context (one JSON object each):
    FP64 CG + Jacobi on 256^2 Poisson, FP64 MG-PCG (Chebyshev 3+3) on 128^3 Poisson, the
    1024^2 obstacle QP (MPRGP, multicolour PGS) and the differentiable solve at 128^3
    (forward with the mixed MG-PCG, adjoint solve and edge gradient).  Complete solves timed
    by CUDA events on the library's stream, operators resident; the two CG workloads also
    run on the oracle (host cores) and report their error against it."""
    import torch
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    def timed(fn, steps, warm=1):
        ts = []
        for i in range(warm + steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            if i >= warm:
                ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    out = {}
    O = None
    if not args.no_cpu:
        import oracle as O

        O.build()

    # -- 256^2 Poisson, FP64 CG + Jacobi, rtol 1e-8 --
    A, b = P.poisson2d_cg(256, 0)
    nb = float(np.linalg.norm(b))
    Am, bv, x = U.SparseMatrix(ctx, A), U.Vector(ctx, b), U.Vector(ctx, n=A.nrows)
    cg = U.ConjugateGradient(ctx, atol=1e-8 * nb)
    cg.set_preconditioner(U.InvDiagPreconditioner(ctx))
    cg.update(Am)

    def solve1():
        x.set(0.0)
        cg.apply(bv, x)

    ms = timed(solve1, max(args.steps, 3))
    st = cg.solution_status()
    rec = {"workload": "FP64 CG + InvDiagPreconditioner, 2D 5-point Poisson 256^2 (n=65536), rtol 1e-8",
           "ms": ms, "iterations": int(st["iterates"]), "us_per_iteration": ms * 1e3 / max(st["iterates"], 1),
           "rel_residual_fp64": float(np.linalg.norm(b - A.matvec(x.numpy())) / nb)}
    if O is not None:
        Ao = O.Matrix(A)
        t0 = time.perf_counter()
        xo, so = O.cg_solve(Ao, b, atol=1e-8 * nb)
        rec["cpu_oracle_ms"] = (time.perf_counter() - t0) * 1e3
        rec["iterations_minus_oracle"] = int(st["iterates"] - so["iterates"])
        rec["rel_err_vs_oracle"] = float(np.linalg.norm(x.numpy() - xo) / np.linalg.norm(xo))
    out["cg_jacobi_poisson2d_256"] = rec
    del Am, bv, x, cg

    # -- 128^3 Poisson, FP64 MG-PCG, 4 levels, Chebyshev 3+3, rtol 1e-10 --
    A, Ps, b = P.poisson3d_mg(128, 4, seed=1)
    nb = float(np.linalg.norm(b))
    Am, bv, x = U.SparseMatrix(ctx, A), U.Vector(ctx, b), U.Vector(ctx, n=A.nrows)
    mg = U.Multigrid(ctx, smoother="chebyshev", pre_smoothing_steps=3, post_smoothing_steps=3)
    mg.set_transfer_operators([U.SparseMatrix(ctx, p) for p in Ps])
    cg = U.ConjugateGradient(ctx, atol=1e-10 * nb)
    cg.set_preconditioner(mg)
    t0 = time.perf_counter()
    cg.update(Am)
    ctx.synchronize()
    setup = (time.perf_counter() - t0) * 1e3

    def solve2():
        x.set(0.0)
        cg.apply(bv, x)

    ms = timed(solve2, max(args.steps // 4, 3))
    st = cg.solution_status()
    rec = {"workload": "FP64 MG-PCG, 3D 7-point Poisson 128^3 (n=2097152), 4 levels, Chebyshev 3+3, Galerkin "
                       "RAP, dense Cholesky coarse, rtol 1e-10",
           "ms": ms, "setup_ms": setup, "iterations": int(st["iterates"]) + 1,
           "rel_residual_fp64": float(np.linalg.norm(b - A.matvec(x.numpy())) / nb)}
    if O is not None:
        Ao = O.Matrix(A)
        omg = O.Multigrid(Ao, Ps, smoother="chebyshev", pre=3, post=3)
        t0 = time.perf_counter()
        xo, so = O.cg_solve(Ao, b, precond="mg", mg=omg, atol=1e-10 * nb)
        rec["cpu_oracle_ms"] = (time.perf_counter() - t0) * 1e3
        rec["iterations_minus_oracle"] = int(st["iterates"] - so["iterates"])
        rec["rel_err_vs_oracle"] = float(np.linalg.norm(x.numpy() - xo) / np.linalg.norm(xo))
    out["mgpcg_fp64_poisson3d_128"] = rec
    del Am, bv, x, cg, mg

    # -- 1024^2 obstacle: as specified (b = -1) and with a free boundary (b = -20 h^2) --
    out["obstacle_1024"] = {
        "as_specified": qp_measure(ctx, 1024, None, 2),
        "free_boundary": qp_measure(ctx, 1024, 20.0, 1, pgs_max_it=2000),
        "note": "PGS on the free-boundary case is capped at 2000 iterations: its per-iteration time is the figure"}

    # -- differentiable solve at 128^3: forward (assembly, hierarchy, mixed MG-PCG to 1e-8),
    #    backward (adjoint solve with the same hierarchy, edge gradient) --
    from utopia_gb300.autograd import DifferentiableGraphSolver

    G, theta, b, _ = P.graph_adjoint(128)
    Ps = P.hierarchy_3d(128, 4)
    ds = DifferentiableGraphSolver(ctx, G, Ps, precision=U.BF16, rtol=1e-8)
    th = U.Vector(ctx, theta, dtype=U.F32)
    bv, x, lam = U.Vector(ctx, b), U.Vector(ctx, n=G.n), U.Vector(ctx, n=G.n)
    g = U.Vector(ctx, np.random.default_rng(6).standard_normal(G.n))
    grad = U.Vector(ctx, n=G.E, dtype=U.F32)
    ms_f = timed(lambda: ds.forward(th, bv, x), 2)

    def backward():
        ds.adjoint(g, lam)
        ds.edge_grad(th, lam, x, grad)

    ms_b = timed(backward, 2)
    out["adjoint_graph_128"] = {
        "workload": "x = A(theta)^-1 b on the 128^3 7-point graph (6,242,304 edges, FP32 theta), mixed MG-PCG "
                    "(4 levels, BF16/FP32 V-cycle, FP64 FCG) at rtol 1e-8",
        "forward_ms": ms_f, "backward_ms": ms_b, "ms": ms_f + ms_b,
        "forward_iterations": int(ds.status["forward"]["iterates"]) + 1,
        "adjoint_iterations": int(ds.status["adjoint"]["iterates"]) + 1,
        "forward_includes": "assembly of A(theta), Galerkin hierarchy and coarse Cholesky, solve",
        "backward_includes": "adjoint solve with the forward pass's hierarchy, edge-gradient kernel"}
    return out


def run_qp(args):
    """Box-constrained QP throughput (one JSON line): the 1024^2 obstacle problem as specified
    (b = -1: every node ends in contact) and with b = -20 h^2 (a free boundary), MPRGP and
    multicolour PGS, plus the per-iteration byte model of MPRGP's CG step."""
    import utopia_gb300 as U

    ctx = U.Context(0)
    N = args.size if args.size != N_GRID else 1024
    out = {"metric": f"box-QP time-to-solution, obstacle {N}^2", "unit": "ms", "higher_is_better": False}
    out["as_specified"] = qp_measure(ctx, N, None, args.steps, eager=args.eager)
    out["free_boundary"] = qp_measure(ctx, N, 20.0, args.steps, eager=args.eager, max_it=args.qp_max_it,
                                      pgs=not args.no_pgs)
    print(json.dumps(out), flush=True)


def run_mmg(args):
    """MonotoneMultigrid on the 2D obstacle problem (5-point Laplacian on an N x N interior grid,
    b = -20 h^2, Gaussian-bump lower bound), 7-level geometric hierarchy: complete solves
    (update + apply: PGS set-up, active-set truncations and Galerkin rebuilds, V-cycles) timed by
    the wall clock around a synchronised call, the GPU MPRGP on the same problem beside it, and
    the oracle's monotone multigrid on the host cores for a bounded number of iterations.  One
    JSON line."""
    import utopia_gb300 as U
    from utopia_gb300 import problems as P

    N = args.size if args.size != N_GRID else 1024
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-20.0 * h * h)
    levels = 7
    Ps = P.hierarchy_2d(N, levels)
    atol, stol = 1e-8 * h * h, 1e-12
    ctx = U.Context(0)
    Am, bv, x = U.SparseMatrix(ctx, A), U.Vector(ctx, b), U.Vector(ctx, n=A.nrows)
    lbv, ubv = U.Vector(ctx, lb), U.Vector(ctx, ub)
    out = {"metric": f"MonotoneMultigrid time-to-solution, obstacle {N}^2", "unit": "ms", "higher_is_better": False,
           "config": {"workload": f"2D obstacle QP {N}x{N} (n={A.nrows}), b=-20h^2, {levels}-level geometric "
                                  "hierarchy, PGS 3+3, Chebyshev3level below the truncated level",
                      "tolerance": f"||P(x-g)-x|| <= {atol:.3g} or ||x - x_old|| <= {stol}"}}
    solvers = {"monotone_mg": lambda: U.MonotoneMultigrid(ctx, max_it=500, atol=atol, stol=stol),
               "mprgp": lambda: U.MPRGP(ctx, max_it=200000, atol=atol)}
    for name, make in solvers.items():
        s = make()
        if name == "monotone_mg":
            s.set_transfer_operators(Ps)
        s.set_box_constraints(lbv, ubv if name == "mprgp" else None)
        times = []
        for i in range(1 + max(1, args.steps)):
            x.set(0.0)
            ctx.synchronize()
            t0 = time.perf_counter()
            s.solve(Am, bv, x)
            ctx.synchronize()
            if i >= 1:
                times.append((time.perf_counter() - t0) * 1e3)
        st = s.solution_status()
        rec = {"ms": float(np.median(times)), "iterations": int(st["iterates"]), "converged": bool(st["converged"]),
               "gradient_norm": float(st["gradient_norm"])}
        if name == "monotone_mg":
            rec["galerkin_assemblies"] = int(s.get("galerkin_assemblies"))
            rec["n_active"] = int(s.get("n_active"))
            rec["ms_per_iteration"] = rec["ms"] / max(rec["iterations"], 1)
            xm = x.numpy()
        out[name] = rec
    out["max_abs_diff_mmg_vs_mprgp"] = float(np.abs(xm - x.numpy()).max())
    if not args.no_cpu:
        import oracle as O

        O.build()
        Ao = O.Matrix(A)
        colour = O.colouring(Ao)[0]
        k = 10
        t0 = time.perf_counter()
        O.monotone_mg_solve(Ao, b, lb, None, Ps, colour=colour, max_it=k + 1, atol=atol, stol=stol)
        per_it = (time.perf_counter() - t0) * 1e3 / k
        out["cpu_baseline"] = {"value": per_it, "unit": "ms/iteration", "kind": "port", "cores": O.max_threads(),
                               "sample": f"the oracle's monotone multigrid, first {k} iterations (set-up included)",
                               "extrapolated_ms": per_it * out["monotone_mg"]["iterations"]}
    out["value"] = out["monotone_mg"]["ms"]
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N_GRID)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the other workloads (256^2 CG, 128^3 MG-PCG, obstacle QP, adjoint) in the default line")
    ap.add_argument("--profile", action="store_true", help="one warm-up and one timed solve only (for ncu)")
    ap.add_argument("--eager", action="store_true",
                    help="launch every kernel individually instead of one graph per solve (ncu does not "
                         "profile kernels inside conditional graph bodies)")
    ap.add_argument("--amg", action="store_true",
                    help="AMG-PCG measurement (algebraic multigrid), one JSON line; not the headline metric")
    ap.add_argument("--mmg", action="store_true",
                    help="MonotoneMultigrid measurement (2D obstacle problem), one JSON line; not the headline metric")
    ap.add_argument("--qp", action="store_true",
                    help="box-constrained QP measurement (MPRGP, multicolour PGS on the 1024^2 obstacle problem)")
    ap.add_argument("--qp-max-it", type=int, default=400000, help="iteration cap of the --qp free-boundary solves")
    ap.add_argument("--no-pgs", action="store_true", help="--qp: MPRGP only")
    ap.add_argument("--cg-jacobi", action="store_true",
                    help="profiling case: four eager iterations of FP64 Jacobi-preconditioned CG, nothing else")
    ap.add_argument("--spmv-only", action="store_true",
                    help="profiling case: FP64 and FP32 products and a BF16 Jacobi sweep of the fine operator, "
                         "two launches each, nothing else")
    ap.add_argument("--transfers", action="store_true",
                    help="profiling case: the BF16 and FP64 restriction and the BF16 prolongation (add form) of "
                         "the fine level to the next, L2 flushed between launches; one JSON line")
    ap.add_argument("--setup", action="store_true",
                    help="the cold path in parts (operator and transfer uploads, hierarchy set-up, first and "
                         "second solve), three repetitions; one JSON line")
    args = ap.parse_args()
    if args.transfers:
        run_transfers(args)
        return
    if args.setup:
        run_setup(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.spmv_only:
        run_spmv_only(args)
        return
    if args.cg_jacobi:
        run_cg_jacobi(args)
        return
    if args.amg:
        run_amg(args)
        return
    if args.mmg:
        run_mmg(args)
        return
    if args.qp:
        run_qp(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)

    import utopia_gb300 as U
    from utopia_gb300 import _abi

    if not os.path.exists(_abi.LIB_PATH):
        from utopia_gb300 import build

        build.build()

    A, Ps, b = make_problem(args.size)
    n, nnz = A.nrows, A.nnz
    nb = float(np.linalg.norm(b))
    ctx = U.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)

    Am = U.SparseMatrix(ctx, A)
    Pm = [U.SparseMatrix(ctx, p) for p in Ps]
    bv = U.Vector(ctx, b)

    def solver(precision, flexible):
        mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                         precision=precision)
        mg.set_transfer_operators(Pm)
        cg = U.ConjugateGradient(ctx, atol=RTOL * nb, flexible=flexible, use_graphs=0 if args.eager else 1)
        cg.set_preconditioner(mg)
        t0 = time.perf_counter()
        cg.update(Am)
        ctx.synchronize()
        return cg, mg, time.perf_counter() - t0

    mixed, mg_mixed, setup_mixed = solver(U.BF16, 1)
    plain, mg_plain, setup_plain = solver(U.F64, 0)
    x = U.Vector(ctx, n=n)

    def timed_solves(cg, k):
        evs = []
        for _ in range(k):
            x.set(0.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            cg.apply(bv, x)
            e.record(stream)
            evs.append((s, e))
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in evs], cg.solution_status()

    steps = 1 if args.profile else args.steps
    warm = 1 if args.profile else args.warmup
    with ClockSampler(local) as clk:
        timed_solves(mixed, warm)
        timed_solves(plain, warm)
        time.sleep(0.3 if not args.profile else 0)  # let the sampler start
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = ctx.launch_count()
        w0 = clk.mark()
        t_mixed, st_mixed = timed_solves(mixed, steps)
        w1 = clk.mark()
        launches = (ctx.launch_count() - l0) // max(steps, 1)
        x_mixed = x.numpy()
        w2 = clk.mark()
        t_plain, st_plain = timed_solves(plain, steps)
        w3 = clk.mark()
        x_plain = x.numpy()
        clk.keep([(w0, w1), (w2, w3)])
    if dist:
        t = torch.tensor([max(t_mixed)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_mixed = float(np.mean(t_mixed))
    ms_plain = float(np.mean(t_plain))
    res_mixed = float(np.linalg.norm(b - A.matvec(x_mixed)) / nb)
    res_plain = float(np.linalg.norm(b - A.matvec(x_plain)) / nb)
    err_mixed_vs_fp64 = float(np.linalg.norm(x_mixed - x_plain) / np.linalg.norm(x_plain))

    # ---- roofline: the FP64 fine-level SpMV, timed alone (the CSR byte model nnz (8 + 4) + 4 (n + 1) + 2 n 8) ----
    hbm, peak_kind = peaks()
    y = U.Vector(ctx, n=n)
    xr = U.Vector(ctx, np.random.default_rng(0).standard_normal(n))

    def time_kernel(fn, reps=30):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            fn()
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e) / reps * 1e-3

    # the FP64 form's dominant kernel is CG's K1, the product fused with (p, Ap): timed as that
    # launch (the dot left on the device), and the store-only product beside it
    dotv = U.Vector(ctx, n=1)
    t_spmv = time_kernel(lambda: Am.apply_dot(xr, y, out=dotv))
    t_store = time_kernel(lambda: Am.apply(xr, y))
    csr_bytes = nnz * (8 + 4) + 4 * (n + 1) + 2 * n * 8
    sell = Am.sell_info()
    moved_bytes = sell["nstored"] * 8 + 2 * n * 8 + 4 * sell["nslices"] * 3
    fp64_ops = sell["nstored"] + n  # one DFMA per stored slot, one per row for the dot
    # the FP64 pipe's rate on this GPU, measured now (FMA chains on every thread; the FP64
    # tensor path beside it)
    dfma = ctx.fp64_rate("dfma")
    dmma = ctx.fp64_rate("dmma")
    fma_peak = dfma / 2
    spmv = {"kernel": "k_sell_spmv<double,double,2,EPI_STORE,XM0,DOT> (product + (x, y))", "us": t_spmv * 1e6,
            "store_only_us": t_store * 1e6,
            "csr_model_gbs": csr_bytes / t_spmv / 1e9, "format_bytes_gbs": moved_bytes / t_spmv / 1e9,
            "csr_model_bytes": csr_bytes, "format_bytes": moved_bytes, "fp64_fma_per_launch": fp64_ops}
    Am.set_format(U.FORMAT_CSR)
    t_csr = time_kernel(lambda: Am.apply(xr, y))
    Am.set_format(U.FORMAT_SELL)
    spmv["csr_kernel_us"] = t_csr * 1e6
    spmv["csr_kernel_gbs"] = csr_bytes / t_csr / 1e9
    # DRAM read+write bytes of one launch of this kernel, from an ncu capture of the 160^3
    # operator (268.8 MB for 28,518,400 nonzeros) scaled by nonzeros (traffic grows with them)
    traffic = 268.8e6 * nnz / 28518400
    roofline = {"bound": "hbm", "achieved": csr_bytes / t_spmv / 1e9, "peak": hbm, "unit": "GB/s",
                "frac": csr_bytes / t_spmv / 1e9 / hbm, "traffic": traffic,
                "format_frac": moved_bytes / t_spmv / 1e9 / hbm,
                "fp64_pipe_frac": fp64_ops / t_spmv / fma_peak,
                "fp64_measured_tflops": {"dfma": dfma / 1e12, "dmma_m8n8k4": dmma / 1e12},
                "kernel": spmv["kernel"], "peak_kind": f"{peak_kind} hbm_gbs (burst copy)",
                "bytes_model": "frac: nnz*(8+4) + 4(n+1) + 2n*8 per launch (the CSR model); format_frac: the "
                               "bytes the diagonal-keyed sliced ELL moves (stored slots x 8 + 2n x 8 + slice "
                               "headers; no column indices)",
                "limit": f"FP64 pipe: fp64_pipe_frac of {fma_peak / 1e9:.0f} G DFMA/s, the DFMA rate measured "
                         "on this GPU in this run (the FP64 tensor path, DMMA, measured beside it)"}
    # the V-cycle's operator in the mixed form: BF16 values, FP32 vectors
    A16 = Am.cast(U.BF16)
    x16, y16 = U.Vector(ctx, np.ones(n, np.float32), dtype=U.F32), U.Vector(ctx, n=n, dtype=U.F32)
    t16 = time_kernel(lambda: A16.apply(x16, y16))
    s16 = A16.sell_info()
    b16 = s16["nstored"] * 2 + 2 * n * 4
    roofline_bf16 = {"kernel": "k_sell_staged<bf16,EPI_STORE> (shared-memory staged sliced ELL)", "us": t16 * 1e6,
                     "format_bytes": b16, "achieved": b16 / t16 / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": b16 / t16 / 1e9 / hbm, "csr_model_gbs": (nnz * 6 + 4 * (n + 1) + 2 * n * 4) / t16 / 1e9}
    del A16

    # ---- e2e through the public C ABI with host buffers: per step, b from pinned host
    # memory to the device, the mixed solve, x back to pinned host memory ----
    hb = torch.from_numpy(b).pin_memory()
    hx = torch.empty(n, dtype=torch.float64).pin_memory()
    b_dev, x_dev = U.Vector(ctx, n=n), U.Vector(ctx, n=n)

    def e2e_step():
        b_dev.upload_from(hb.data_ptr())
        x_dev.set(0.0)
        mixed.apply(b_dev, x_dev)
        x_dev.download_to(hx.data_ptr())

    for _ in range(warm):
        e2e_step()
    e2e_t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    assert np.linalg.norm(b - A.matvec(hx.numpy())) <= RTOL * nb * 1.0001
    e2e = {"value": float(np.mean(e2e_t)) * 1e3, "unit": "ms", "h2d_bytes_per_step": int(b.nbytes),
           "d2h_bytes_per_step": int(n * 8),
           "includes": "host-timed ConjugateGradient.apply through the C ABI: b copied from pinned host memory, "
                       "solve, x copied back; operator and hierarchy resident (set up once)"}

    # ---- the cold path: operator and transfers from host arrays, hierarchy set-up, solve ----
    def cold_once():
        t0 = time.perf_counter()
        A_d = U.SparseMatrix(ctx, A)
        P_d = [U.SparseMatrix(ctx, p) for p in Ps]
        b_d = U.Vector(ctx, b)
        mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                         precision=U.BF16)
        mg.set_transfer_operators(P_d)
        cg = U.ConjugateGradient(ctx, atol=RTOL * nb, flexible=1)
        cg.set_preconditioner(mg)
        x_d = U.Vector(ctx, n=n)
        cg.solve(A_d, b_d, x_d)
        x_d.numpy()
        return time.perf_counter() - t0

    cold_ms = min(cold_once() for _ in range(1 if args.profile else 2)) * 1e3
    cold_h2d = (A.rowptr.nbytes + A.colidx.nbytes + A.values.nbytes + b.nbytes
                + sum(p.rowptr.nbytes + p.colidx.nbytes + p.values.nbytes for p in Ps))

    others = None
    if rank == 0 and not args.no_extra and not args.profile:
        others = extra_workloads(ctx, args, stream)

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu and not args.profile:
        O, Aor, mgor, setup_s = oracle_setup(A, Ps)
        dt, st, x_or = oracle_solve(O, Aor, mgor, b, with_x=True)
        cpu = {"value": dt * 1e3, "unit": "ms", "cores": O.max_threads(), "kind": "port",
               "sample": f"one complete FP64 MG-PCG solve of the same {args.size}^3 problem on the oracle "
                         f"({st['iterates'] + 1} iterations); hierarchy set-up {setup_s:.1f} s untimed"}
        # the GPU results against the oracle's solve of the same problem: Galerkin structure
        # of every level, iteration counts and solutions
        same_structure = True
        for lev in range(mg_plain.n_levels() - 1):
            rp, ci, _ = mg_plain.level_matrix(lev).csr()
            orp, oci, _ = mgor.level_matrix(lev).arrays()
            same_structure &= bool(np.array_equal(rp, orp) and np.array_equal(ci, oci))
        nrm = float(np.linalg.norm(x_or))
        parity = {"oracle_iterations": st["iterates"] + 1,
                  "fp64_rel_err_vs_oracle": float(np.linalg.norm(x_plain - x_or) / nrm),
                  "mixed_rel_err_vs_oracle": float(np.linalg.norm(x_mixed - x_or) / nrm),
                  "fp64_iterations_minus_oracle": int(st_plain["iterates"] - st["iterates"]),
                  "galerkin_structure_identical": same_structure, "levels": mg_plain.n_levels()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms_mixed, "unit": "ms", "n_gpus": world, "steps": steps,
            "warmup": warm, "ms_per_step": ms_mixed, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32/bf16", "data": "synthetic",
            "config": {"workload": f"lognormal diffusion -div(k grad u), {args.size}^3 (n={n}, nnz={nnz}), "
                                   "MG-PCG 5 levels Jacobi(0.8) 2+2, Galerkin RAP, dense Cholesky 12^3",
                       "grid": args.size, "tolerance": f"||r|| <= {RTOL} ||b|| (FP64)",
                       "timed": "solve phase per step (hierarchy built before the timed region)",
                       "l2": "inputs larger than L2 (FP64 operator 395 MB), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "mixed": {"ms": ms_mixed, "iterations": st_mixed["iterates"] + 1, "rel_residual_fp64": res_mixed,
                      "rel_err_vs_fp64": err_mixed_vs_fp64, "setup_ms": setup_mixed * 1e3,
                      "precision": "BF16-stored level matrices, FP32 V-cycle, FP64 FCG"},
            "fp64": {"ms": ms_plain, "iterations": st_plain["iterates"] + 1, "rel_residual_fp64": res_plain,
                     "setup_ms": setup_plain * 1e3},
            "speedup_mixed_vs_fp64": ms_plain / ms_mixed,
            "speedup_fp64_gpu_vs_cpu": (cpu["value"] / ms_plain) if cpu else None,
            "parity_vs_oracle": parity,
            "spmv": spmv,
            "roofline": roofline,
            "roofline_bf16_spmv": roofline_bf16,
            "e2e": e2e,
            "cold_path": {"ms": cold_ms, "h2d_bytes": int(cold_h2d),
                          "includes": "CSR + transfer upload from pageable host arrays, Galerkin hierarchy, "
                                      "coarse Cholesky, solve, download"},
            "cpu_baseline": cpu,
            "other_workloads": others,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
