"""BiCGStab through the C ABI against the oracle's restatement of utopia_BiCGStab_impl.hpp:44-250:
unpreconditioned and Jacobi-preconditioned on a nonsymmetric convection-diffusion operator, and
multigrid-preconditioned on the lognormal diffusion operator."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def gpu_bicgstab(ctx, A, b, atol, prec=None):
    s = U.BiCGStab(ctx, atol=atol, max_it=3000)
    if prec is not None:
        s.set_preconditioner(prec)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    return x.numpy(), s.solution_status()


@pytest.mark.parametrize("pc", ["none", "invdiag"])
def test_bicgstab_convection_diffusion(ctx, oracle, pc):
    A = P.convection_diffusion_2d(96, 20.0)
    b = np.random.default_rng(5).uniform(-1, 1, A.nrows)
    atol = 1e-10 * np.linalg.norm(b)
    x, st = gpu_bicgstab(ctx, A, b, atol, U.InvDiagPreconditioner(ctx) if pc == "invdiag" else None)
    xr, ost = oracle.bicgstab_solve(oracle.Matrix(A), b, precond=pc, atol=atol, max_it=3000)
    assert st["converged"] and ost["converged"]
    assert abs(st["iterates"] - ost["iterates"]) <= max(1, ost["iterates"] // 20)
    assert np.linalg.norm(b - A.matvec(x)) <= atol * 1.0001
    assert np.linalg.norm(x - xr) <= 1e-7 * np.linalg.norm(xr)


def test_bicgstab_multigrid_preconditioned(ctx, oracle):
    A = P.lognormal_diffusion_3d(24, 5)[0]
    Ps = P.hierarchy_3d(24, 3)
    b = np.random.default_rng(6).uniform(-1, 1, A.nrows)
    atol = 1e-10 * np.linalg.norm(b)
    mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2)
    mg.set_transfer_operators(Ps)
    x, st = gpu_bicgstab(ctx, A, b, atol, mg)
    Am = oracle.Matrix(A)
    omg = oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
    xr, ost = oracle.bicgstab_solve(Am, b, precond="mg", mg=omg, atol=atol, max_it=3000)
    assert st["converged"] and ost["converged"]
    assert abs(st["iterates"] - ost["iterates"]) <= 1
    assert np.linalg.norm(b - A.matvec(x)) <= atol * 1.0001
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)
