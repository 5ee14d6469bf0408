"""Parity at the workloads' full sizes: the GPU path through the C ABI against the oracle on
the same seeded inputs.

* 192^3 lognormal diffusion (n = 7,077,888), plain FP64 MG-PCG (5 levels, Jacobi 0.8 2+2,
  Galerkin RAP, dense Cholesky 12^3) at atol = 1e-10 ||b||: Galerkin rowptr/colidx of every
  level identical, iteration count within 1, x within 1e-9 relative L2.  The mixed form
  (BF16-stored FP32 V-cycle in FP64 flexible CG) at 1e-8: residual checked in FP64 and its
  error against the FP64 oracle solution bounded.
* The 1024^2 obstacle QP exactly as specified (5-point Laplacian, b = -1, seed 3): MPRGP's
  active set bit-exact against the oracle's and multicolour projected Gauss-Seidel's
  converged active set equal to MPRGP's.  With b = -1 on the unscaled Laplacian every node is
  active (the unconstrained minimiser reaches about -7.7e4); the active fraction is printed.
* The same obstacle at 512^2 with b = -20 h^2 (a free boundary through the domain): MPRGP
  active set bit-exact, x within 1e-9, and the PGS active set equal to it.
* Multigrid as a stand-alone solver (utopia_Multigrid.hpp:162-238): the iterates after
  1..4 cycles against the oracle's.
"""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def lognormal192():
    return P.lognormal_mg(192, 5, seed=2)


def test_lognormal192_fp64_matches_oracle(ctx, oracle, lognormal192):
    A, Ps, b = lognormal192
    atol = 1e-10 * np.linalg.norm(b)
    Am = oracle.Matrix(A)
    omg = oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
    xo, so = oracle.cg_solve(Am, b, precond="mg", mg=omg, atol=atol)
    mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2)
    mg.set_transfer_operators(Ps)
    s = U.ConjugateGradient(ctx, atol=atol)
    s.set_preconditioner(mg)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    assert mg.n_levels() == 5
    for l in range(mg.n_levels() - 1):
        rp, ci, v = mg.level_matrix(l).csr()
        orp, oci, ov = omg.level_matrix(l).arrays()
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci), f"level {l} structure"
        np.testing.assert_allclose(v, ov, rtol=1e-12, atol=1e-14 * np.abs(ov).max())
    st = s.solution_status()
    err = rel(x.numpy(), xo)
    print(f"192^3 FP64: iterations {st['iterates']} (oracle {so['iterates']}), rel. error vs oracle {err:.3e}")
    assert abs(st["iterates"] - so["iterates"]) <= 1
    assert err <= 1e-9


def test_lognormal192_mixed_against_fp64_oracle(ctx, oracle, lognormal192):
    A, Ps, b = lognormal192
    nb = np.linalg.norm(b)
    Am = oracle.Matrix(A)
    omg = oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
    xo, _ = oracle.cg_solve(Am, b, precond="mg", mg=omg, atol=1e-12 * nb)
    mg = U.Multigrid(ctx, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                     precision=U.BF16)
    mg.set_transfer_operators(Ps)
    s = U.ConjugateGradient(ctx, atol=1e-8 * nb, flexible=1)
    s.set_preconditioner(mg)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xg = x.numpy()
    res = np.linalg.norm(b - A.matvec(xg)) / nb
    err = rel(xg, xo)
    print(f"192^3 mixed: iterations {s.solution_status()['iterates']}, FP64 residual {res:.3e}, "
          f"rel. error vs FP64 oracle {err:.3e}")
    assert res <= 1e-8
    assert err <= 1e-6


def _mprgp(ctx, A, b, lb, ub, **kw):
    s = U.MPRGP(ctx, **kw)
    s.set_box_constraints(U.Vector(ctx, lb), U.Vector(ctx, ub))
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    return x.numpy(), s.solution_status()


def _pgs(ctx, A, b, lb, ub, **kw):
    s = U.ProjectedGaussSeidel(ctx, **kw)
    s.set_box_constraints(U.Vector(ctx, lb), U.Vector(ctx, ub))
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    return x.numpy(), s.solution_status()


def test_obstacle1024_as_specified(ctx, oracle):
    """b = -1, projected-gradient norm 1e-8."""
    A, b, lb, ub = P.obstacle_qp(1024, seed=3, rhs=-1.0)
    Am = oracle.Matrix(A)
    xo, so = oracle.mprgp_solve(Am, b, lb, ub, atol=1e-8, rtol=1e-30, max_it=100000)
    xg, st = _mprgp(ctx, A, b, lb, ub, atol=1e-8, rtol=1e-30, max_it=100000)
    assert st["converged"] and so["converged"]
    assert st["iterates"] == so["iterates"]
    assert np.array_equal(xg == lb, xo == lb)
    assert np.array_equal(xg, xo)
    frac = float((xg == lb).mean())
    print(f"1024^2 obstacle, b = -1: MPRGP {st['iterates']} iteration(s), active fraction {frac:.6f}")
    assert oracle.projected_gradient_norm(Am, b, lb, ub, xg) <= 1e-8
    xp, sp = _pgs(ctx, A, b, lb, ub, atol=1e-8, max_it=100000, projected_gradient_stop=1)
    assert sp["converged"]
    assert np.array_equal(xp == lb, xg == lb)
    assert oracle.projected_gradient_norm(Am, b, lb, ub, xp) <= 1e-8


def test_obstacle512_free_boundary(ctx, oracle):
    """b = -20 h^2: about a third of the nodes in contact; MPRGP bit-exact active set against
    the oracle, multicolour PGS (stopped at ||x - x_old|| <= 1e-12) on the same active set."""
    N = 512
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-20 * h * h)
    atol = 1e-8 * h * h
    Am = oracle.Matrix(A)
    xo, so = oracle.mprgp_solve(Am, b, lb, ub, atol=atol, rtol=1e-30, max_it=200000)
    xg, st = _mprgp(ctx, A, b, lb, ub, atol=atol, rtol=1e-30, max_it=200000)
    assert st["converged"] and so["converged"]
    frac = float((xg == lb).mean())
    print(f"512^2 obstacle, b = -20h^2: MPRGP {st['iterates']} iterations (oracle {so['iterates']}), "
          f"active fraction {frac:.4f}")
    assert np.array_equal(xg == lb, xo == lb)
    assert rel(xg, xo) <= 1e-9
    assert abs(st["iterates"] - so["iterates"]) <= max(2, 0.02 * so["iterates"])
    xp, sp = _pgs(ctx, A, b, lb, ub, stol=1e-12, max_it=400000)
    assert sp["converged"]
    assert np.array_equal(xp == lb, xo == lb)
    assert rel(xp, xo) <= 1e-9


@pytest.mark.parametrize("smoother", ["chebyshev", "jacobi", "point_jacobi"])
def test_multigrid_standalone_iterates(ctx, oracle, smoother):
    A, Ps, b = P.poisson3d_mg(32, 3, seed=1)
    Am = oracle.Matrix(A)
    kw = dict(pre=3, post=3) if smoother == "chebyshev" else dict(pre=2, post=2)
    omg = oracle.Multigrid(Am, Ps, smoother=smoother, **kw)
    for k in (1, 2, 3, 4):
        xo, so = omg.solve(b, atol=0.0, rtol=0.0, max_it=k)
        mg = U.Multigrid(ctx, smoother=smoother, pre_smoothing_steps=kw["pre"], post_smoothing_steps=kw["post"],
                         atol=0.0, rtol=0.0, max_it=k)
        mg.set_transfer_operators(Ps)
        x = U.Vector(ctx, n=A.nrows)
        mg.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
        st = mg.solution_status()
        assert st["iterates"] == so["iterates"]
        assert rel(x.numpy(), xo) <= 1e-12
        np.testing.assert_allclose(st["gradient_norm"], so["gradient_norm"], rtol=1e-10)
