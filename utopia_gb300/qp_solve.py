"""qp_solve: a box-constrained QP with a contact transformation, read from files, solved on one GPU.

The counterpart of the reference's monotone-multigrid QP app (MGQPSolveApp::run_mg_qr without
the QR factors, utopia/apps/qp_solve/utopia_qp_solve.cpp:90-330): from a directory it reads
(PETSc binary, file names as the reference's defaults) the operator `A`, right-hand side `rhs`,
initial guess `x`, the contact rotation `Rot`, the bounds `lb` and `ub` and the interpolations
`I1 .. I<n>` (coarse -> fine), builds the rotated system

    A' = Rot A Rot,   rhs' = Rot rhs,   x' = Rot x,   I<n>' = Rot I<n>

(create_linear_system; the last interpolation becomes the truncated fine-level transfer), solves
min 1/2 x'^T A' x' - rhs'^T x' subject to lb <= x' <= ub with the monotone multigrid (projected
Gauss-Seidel smoothing, max_it 40, 3 + 3 steps by default) and writes x = Rot x' (report_result).
`--solver` can name another box-constrained solver for the rotated system (mprgp, pgs,
semismooth_newton; these need no interpolations).  One JSON line on stdout.

    python -m utopia_gb300.qp_solve --dir D [--out x.bin] [--oracle x_ref.bin] [--solver monotone_mg]
        [--n_interpolators 4] [--interp_index_offset 1] [--max_it 40] [--pre 3] [--post 3]
        [--atol 1e-9] [--stol 1e-11] [--active_set_tol 0] [--device 0]
    python -m utopia_gb300.qp_solve --dir D --solver shifted_penalty [--use_trafo 1] [--out out.bin]
        [--penalty_parameter 1e4] [--penalty_parameter_max 0] [--penalty_parameter_factor 1.5]
        [--linear_rtol 1e-12] [--max_it 1000] [--stol 1e-11]

`--solver shifted_penalty` is the reference's other QP app (QPSolveApp::solve_with_shifted_penalty,
utopia_qp_solve.cpp:61-107, registered as qp_solve): it reads `A`, `T`, `O`, `rhs`, `upper_bound` and
`is_contact`, enforces x <= upper_bound in the transformed space O^T (T x) (`--use_trafo 0`: in x
itself) with the shifted-penalty solver from x = 0 and writes x (default `out.bin`, as the app's
output_path).

The reference's QR variant (MGQPSolveApp with ProjectedGaussSeidelQR) is unreachable in its app:
Problem::read keeps a local `use_QR = false`, so Q and R are never read and use_QR_mg() is false.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

import utopia_gb300 as U
from utopia_gb300.ls_solve import read_matrix, read_vector


def rotate_system(A, rhs, x, Rot, I_fine):
    """create_linear_system (without Q): Rot A Rot, Rot rhs, Rot x, and Rot I for the fine transfer."""
    ctx = A.ctx
    Ar = Rot.matmul(A).matmul(Rot)
    n = A.nrows
    rr, xr = U.Vector(ctx, n=n), U.Vector(ctx, n=n)
    Rot.apply(rhs, rr)
    Rot.apply(x, xr)
    Ir = Rot.matmul(I_fine) if I_fine is not None else None
    return Ar, rr, xr, Ir


def shifted_penalty_app(a, path) -> dict:
    """QPSolveApp::solve_with_shifted_penalty (utopia_qp_solve.cpp:61-107)."""
    t0 = time.perf_counter()
    ctx = U.Context(a.device)
    A = read_matrix(ctx, path("A"))
    T = read_matrix(ctx, path("T"))
    O = read_matrix(ctx, path("O"))
    rhs = read_vector(ctx, path("rhs"))
    ub = read_vector(ctx, path("upper_bound"))
    is_contact = read_vector(ctx, path("is_contact"))  # required by Problem::read, unused by the solve
    n = A.nrows
    for v, what in ((rhs, "rhs"), (ub, "upper_bound"), (is_contact, "is_contact")):
        if len(v) != n:
            raise ValueError(f"{what} has {len(v)} entries, A has {n} rows")
    t_read = time.perf_counter() - t0
    t1 = time.perf_counter()
    solver = U.ShiftedPenaltyQPSolver(ctx, max_it=a.max_it if a.max_it is not None else 1000, stol=a.stol,
                                      penalty_parameter=a.penalty_parameter,
                                      penalty_parameter_max=a.penalty_parameter_max,
                                      penalty_parameter_factor=a.penalty_parameter_factor,
                                      linear_rtol=a.linear_rtol)
    if a.use_trafo:
        solver.set_transform(T, O)
    solver.set_box_constraints(None, ub)
    x = U.Vector(ctx, n=n)
    solver.solve(A, rhs, x)
    ctx.synchronize()
    t_solve = time.perf_counter() - t1
    st = solver.solution_status()
    xh = x.numpy()
    w = x
    if a.use_trafo:  # the constrained quantity O^T (T x)
        t = U.Vector(ctx, n=n)
        T.apply(x, t)
        w = U.Vector(ctx, n=n)
        O.transpose().apply(t, w)
    out = {"app": "qp_solve", "solver": "shifted_penalty", "n": n, "nnz": A.nnz, "converged": bool(st["converged"]),
           "iterations": int(st["iterates"]), "inner_iterations": int(st["spmv_count"]),
           "violation": float(max(0.0, (w.numpy() - ub.numpy()).max(initial=0.0))),
           "read_s": t_read, "solve_s": t_solve}
    if a.oracle:
        xo = read_vector(ctx, a.oracle).numpy()
        out["error_vs_oracle"] = float(np.linalg.norm(xh - xo) / max(np.linalg.norm(xo), 1e-300))
    dest = a.out or "out.bin"
    (x.write_raw if dest.endswith(".raw") else x.write_petsc)(dest)
    print(json.dumps(out), flush=True)
    return out


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(prog="qp_solve", description=__doc__.split("\n")[0])
    ap.add_argument("--dir", required=True)
    for name in ("A", "rhs", "x", "Rot", "lb", "ub", "I", "T", "O", "upper_bound", "is_contact"):
        ap.add_argument("--" + name, default="", help=f"path of {name} (default: <dir>/{name})")
    ap.add_argument("--n_interpolators", type=int, default=4)
    ap.add_argument("--interp_index_offset", type=int, default=1)
    ap.add_argument("--solver", default="monotone_mg",
                    choices=["monotone_mg", "mprgp", "pgs", "semismooth_newton", "shifted_penalty"])
    ap.add_argument("--use_trafo", type=int, default=1, help="shifted_penalty: constrain O^T (T x)")
    ap.add_argument("--penalty_parameter", type=float, default=1e4)
    ap.add_argument("--penalty_parameter_max", type=float, default=0.0, help="0: = penalty_parameter")
    ap.add_argument("--penalty_parameter_factor", type=float, default=1.5)
    ap.add_argument("--linear_rtol", type=float, default=1e-12)
    ap.add_argument("--max_it", type=int, default=None, help="40 (shifted_penalty: 1000)")
    ap.add_argument("--pre", type=int, default=3)
    ap.add_argument("--post", type=int, default=3)
    ap.add_argument("--smoother", default="chebyshev", choices=list(U.SMOOTHERS))
    ap.add_argument("--atol", type=float, default=1e-9)
    ap.add_argument("--stol", type=float, default=1e-11)
    ap.add_argument("--active_set_tol", type=float, default=0.0)
    ap.add_argument("--oracle", default="")
    ap.add_argument("--out", default="")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)

    def path(name):
        return getattr(a, name) or os.path.join(a.dir, name)

    if a.solver == "shifted_penalty":
        return shifted_penalty_app(a, path)
    if a.max_it is None:
        a.max_it = 40
    t0 = time.perf_counter()
    ctx = U.Context(a.device)
    A = read_matrix(ctx, path("A"))
    rhs = read_vector(ctx, path("rhs"))
    x0 = read_vector(ctx, path("x"))
    Rot = read_matrix(ctx, path("Rot"))
    lb = read_vector(ctx, path("lb"))
    ub = read_vector(ctx, path("ub"))
    Is = []
    if a.solver == "monotone_mg":
        base = path("I")
        Is = [read_matrix(ctx, base + str(l + a.interp_index_offset)) for l in range(a.n_interpolators)]
    n = A.nrows
    for v, what in ((rhs, "rhs"), (x0, "x"), (lb, "lb"), (ub, "ub")):
        if len(v) != n:
            raise ValueError(f"{what} has {len(v)} entries, A has {n} rows")
    t_read = time.perf_counter() - t0

    t1 = time.perf_counter()
    Ar, rr, xr, Ir = rotate_system(A, rhs, x0, Rot, Is[-1] if Is else None)
    if a.solver == "monotone_mg":
        solver = U.MonotoneMultigrid(ctx, smoother=a.smoother, max_it=a.max_it, pre_smoothing_steps=a.pre,
                                     post_smoothing_steps=a.post, atol=a.atol, stol=a.stol,
                                     active_set_tol=a.active_set_tol)
        solver.set_transfer_operators(Is[:-1] + [Ir])
    elif a.solver == "mprgp":
        solver = U.MPRGP(ctx, max_it=a.max_it, atol=a.atol)
    elif a.solver == "pgs":
        solver = U.ProjectedGaussSeidel(ctx, max_it=a.max_it, stol=a.stol)
    else:
        solver = U.SemismoothNewton(ctx, max_it=a.max_it, stol=a.stol)
    solver.set_box_constraints(lb, ub)
    solver.solve(Ar, rr, xr)
    x = U.Vector(ctx, n=n)
    Rot.apply(xr, x)  # report_result: x = Rot x'
    ctx.synchronize()
    t_solve = time.perf_counter() - t1

    st = solver.solution_status()
    xh, xrh, lbh, ubh = x.numpy(), xr.numpy(), lb.numpy(), ub.numpy()
    g = U.Vector(ctx, n=n)
    Ar.residual(rr, xr, g)  # -g' = rhs' - A' x'
    gh = g.numpy()
    crit = float(np.linalg.norm(np.clip(xrh + gh, lbh, ubh) - xrh))
    out = {"app": "qp_solve", "solver": a.solver, "n": n, "nnz": A.nnz, "converged": bool(st["converged"]),
           "iterations": int(st["iterates"]), "criticality": crit,
           "n_active": int(np.count_nonzero((xrh <= lbh) | (xrh >= ubh))),
           "bound_violation": float(max(0.0, (lbh - xrh).max(initial=0.0), (xrh - ubh).max(initial=0.0))),
           "read_s": t_read, "solve_s": t_solve}
    if a.oracle:
        xo = read_vector(ctx, a.oracle).numpy()
        out["error_vs_oracle"] = float(np.linalg.norm(xh - xo) / max(np.linalg.norm(xo), 1e-300))
    if a.out:
        (x.write_raw if a.out.endswith(".raw") else x.write_petsc)(a.out)
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    sys.exit(0 if main()["converged"] else 1)
