"""ls_solve: solve A x = b read from files on one GPU.

The counterpart of the reference's ls_solve app (utopia/apps/ls_solve/utopia_ls_solve.cpp:64-150):
A and b are read from files (PETSc binary, or raw CRS: a directory with rowptr.raw, colidx.raw,
values.raw, or the path of its rowptr.raw; raw vectors end in .raw), optionally rescaled by the
inverse diagonal, solved with conjugate gradients preconditioned by Jacobi or by the algebraic
multigrid (use_amg; amg_as_preconditioner=false runs the multigrid alone), and x is written to
`out` (PETSc binary unless it ends in .raw).  With `oracle` the error against that solution is
reported.  One JSON line on stdout.

    python -m utopia_gb300.ls_solve -A A.bin -b rhs.bin [-P P.bin] [--oracle x.bin] [--out x.bin]
        [--use_amg] [--amg_as_preconditioner 0|1] [--rescale_with_diag] [--atol 1e-10] [--rtol 0]
        [--max_it 1000] [--n_levels 0] [--device 0]

The reference's KSP, block-matrix and Matlab-output options have no counterpart here.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

import utopia_gb300 as U


def _is_raw_crs(path: str) -> bool:
    return os.path.isdir(path) or os.path.basename(path) == "rowptr.raw"


def read_matrix(ctx, path: str, index_bytes=4, value_bytes=8):
    if _is_raw_crs(path):
        d = path if os.path.isdir(path) else os.path.dirname(path)
        return U.read_raw_crs(ctx, d, index_bytes, value_bytes)
    return U.read_petsc_matrix(ctx, path)


def read_vector(ctx, path: str, value_bytes=8):
    if path.endswith(".raw"):
        return U.read_raw_vector(ctx, path, value_bytes)
    return U.read_petsc_vector(ctx, path)


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(prog="ls_solve", description=__doc__.split("\n")[0])
    ap.add_argument("-A", required=True)
    ap.add_argument("-b", default="")
    ap.add_argument("-P", default="", help="matrix the Jacobi preconditioner takes its diagonal from")
    ap.add_argument("--oracle", default="")
    ap.add_argument("--out", default="")
    ap.add_argument("--use_amg", action="store_true")
    ap.add_argument("--amg_as_preconditioner", type=int, default=1)
    ap.add_argument("--rescale_with_diag", action="store_true")
    ap.add_argument("--atol", type=float, default=1e-10)
    ap.add_argument("--rtol", type=float, default=0.0)
    ap.add_argument("--max_it", type=int, default=1000)
    ap.add_argument("--n_levels", type=int, default=0)
    ap.add_argument("--index_bytes", type=int, default=4)
    ap.add_argument("--value_bytes", type=int, default=8)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)

    t0 = time.perf_counter()
    ctx = U.Context(a.device)
    A = read_matrix(ctx, a.A, a.index_bytes, a.value_bytes)
    n = A.nrows
    if a.b:
        b = read_vector(ctx, a.b, a.value_bytes)
    else:  # "b is undefined, using vector of ones"
        b = U.Vector(ctx, np.ones(n))
    Pm = read_matrix(ctx, a.P, a.index_bytes, a.value_bytes) if a.P else None
    t_read = time.perf_counter() - t0
    if a.rescale_with_diag:  # A <- D^-1 A, b <- D^-1 b
        rp, ci, v = A.csr()
        d = np.zeros(n)
        rows = np.repeat(np.arange(n), np.diff(rp))
        d[rows[ci == rows]] = v[ci == rows]
        v = v / d[rows]
        A.update_values(v)
        b = U.Vector(ctx, b.numpy() / d)

    rhs_norm = float(np.linalg.norm(b.numpy()))
    atol = max(a.atol, a.rtol * rhs_norm)
    x = U.Vector(ctx, n=n)
    t1 = time.perf_counter()
    if a.use_amg and not a.amg_as_preconditioner:
        solver = U.AlgebraicMultigrid(ctx, n_levels=a.n_levels, atol=atol, rtol=0.0, max_it=a.max_it)
        solver.update(A)
        solver.apply(b, x)
    else:
        solver = U.ConjugateGradient(ctx, atol=atol, max_it=a.max_it)
        pc = U.AlgebraicMultigrid(ctx, n_levels=a.n_levels) if a.use_amg else U.InvDiagPreconditioner(ctx)
        solver.set_preconditioner(pc)
        solver.update(A)
        if Pm is not None and not a.use_amg:
            pc.update(Pm)
        solver.apply(b, x)
    ctx.synchronize()
    t_solve = time.perf_counter() - t1
    st = solver.solution_status()
    xh = x.numpy()
    r = U.Vector(ctx, n=n)
    A.residual(b, x, r)
    out = {"app": "ls_solve", "n": n, "nnz": A.nnz, "converged": bool(st["converged"]),
           "iterations": int(st["iterates"]), "gradient_norm": float(st["gradient_norm"]),
           "read_s": t_read, "solve_s": t_solve,
           "solver": ("amg" if a.use_amg and not a.amg_as_preconditioner else
                      "cg+amg" if a.use_amg else "cg+jacobi")}
    out["residual_norm"] = float(r.norm2())
    if a.oracle:
        xo = read_vector(ctx, a.oracle, a.value_bytes).numpy()
        out["error_vs_oracle"] = float(np.linalg.norm(xh - xo) / max(np.linalg.norm(xo), 1e-300))
    if a.out:
        (x.write_raw if a.out.endswith(".raw") else x.write_petsc)(a.out)
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    sys.exit(0 if main()["converged"] else 1)
