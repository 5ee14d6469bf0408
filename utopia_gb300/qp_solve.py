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

The reference's QR variant (ProjectedGaussSeidelQR with the Q and R factors) and the shifted-penalty
QP app (ShiftedPenaltyQPSolver) have no counterpart here.
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


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(prog="qp_solve", description=__doc__.split("\n")[0])
    ap.add_argument("--dir", required=True)
    for name in ("A", "rhs", "x", "Rot", "lb", "ub", "I"):
        ap.add_argument("--" + name, default="", help=f"path of {name} (default: <dir>/{name})")
    ap.add_argument("--n_interpolators", type=int, default=4)
    ap.add_argument("--interp_index_offset", type=int, default=1)
    ap.add_argument("--solver", default="monotone_mg",
                    choices=["monotone_mg", "mprgp", "pgs", "semismooth_newton"])
    ap.add_argument("--max_it", type=int, default=40)
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
