"""AlgebraicMultigrid (greedy agglomeration + Galerkin hierarchy) through the C ABI against the
oracle: identical aggregates on every level, identical coarse-operator structure, and AMG-
preconditioned CG with the oracle's iteration count and solution."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu

CASES = {
    "laplace1d_dirichlet": (lambda: P.laplacian_1d_dirichlet(100), dict(n_levels=6)),
    "lognormal24": (lambda: P.lognormal_diffusion_3d(24, 5)[0], dict(n_levels=0, max_coarse_rows=2000)),
    "random_graph": (lambda: P.random_spd_graph(20000, 4, 1), dict(n_levels=0, max_coarse_rows=2000)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_amg_hierarchy_matches_oracle(ctx, oracle, name):
    make, kw = CASES[name]
    A = make()
    Am = oracle.Matrix(A)
    Ps, parents = oracle.amg_hierarchy(Am, **kw)
    amg = U.AlgebraicMultigrid(ctx, smoother="chebyshev", **kw)
    M = U.SparseMatrix(ctx, A)
    amg.update(M)
    assert amg.n_levels() == len(Ps) + 1
    for l, ref in enumerate(parents):
        got, nc = amg.parent(l)
        np.testing.assert_array_equal(got, ref)
        assert nc == Ps[len(Ps) - 1 - l].ncols
    omg = oracle.Multigrid(Am, Ps, smoother="chebyshev")
    for l in range(amg.n_levels()):
        G = amg.level_matrix(l)
        rp, ci, v = G.csr()
        orp, oci, ov = omg.level_matrix(l).arrays()
        np.testing.assert_array_equal(rp, orp)
        np.testing.assert_array_equal(ci, oci)
        np.testing.assert_allclose(v, ov, rtol=1e-12, atol=1e-12 * np.abs(ov).max())


def test_reference_amg_1d_case(ctx, oracle):
    """utopia/tests/utopia_AMGTest.cpp:36-110 (1D Laplacian, 100 dofs, identity boundary rows,
    b = 2 with 0 on the boundary, 6 levels, atol 1e-6, ||r||_1 < 1e-5), with Chebyshev3level
    smoothing and the hierarchy as the CG preconditioner (the reference smooths with ILU)."""
    A = P.laplacian_1d_dirichlet(100)
    b = np.full(100, 2.0)
    b[0] = b[-1] = 0.0
    amg = U.AlgebraicMultigrid(ctx, smoother="chebyshev", n_levels=6, pre_smoothing_steps=3,
                               post_smoothing_steps=3)
    cg = U.ConjugateGradient(ctx, atol=1e-6, max_it=100)
    cg.set_preconditioner(amg)
    x = U.Vector(ctx, n=100)
    cg.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = cg.solution_status()
    assert st["converged"] and np.abs(b - A.matvec(x.numpy())).sum() < 1e-5
    Am = oracle.Matrix(A)
    Ps, _ = oracle.amg_hierarchy(Am, n_levels=6)
    _, ost = oracle.cg_solve(Am, b, precond="mg", mg=oracle.Multigrid(Am, Ps, smoother="chebyshev"), atol=1e-6,
                             max_it=100)
    assert abs(st["iterates"] - ost["iterates"]) <= 1


@pytest.mark.parametrize("name", ["lognormal24", "random_graph"])
def test_amg_pcg_matches_oracle(ctx, oracle, name):
    make, kw = CASES[name]
    A = make()
    b = np.random.default_rng(0).uniform(-1, 1, A.nrows)
    atol = 1e-10 * np.linalg.norm(b)
    amg = U.AlgebraicMultigrid(ctx, smoother="chebyshev", pre_smoothing_steps=2, post_smoothing_steps=2, **kw)
    cg = U.ConjugateGradient(ctx, atol=atol, max_it=500)
    cg.set_preconditioner(amg)
    x = U.Vector(ctx, n=A.nrows)
    cg.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = cg.solution_status()
    Am = oracle.Matrix(A)
    Ps, _ = oracle.amg_hierarchy(Am, **kw)
    omg = oracle.Multigrid(Am, Ps, smoother="chebyshev", pre=2, post=2)
    xr, ost = oracle.cg_solve(Am, b, precond="mg", mg=omg, atol=atol, max_it=500)
    assert st["converged"] and ost["converged"]
    assert abs(st["iterates"] - ost["iterates"]) <= 1
    xg = x.numpy()
    assert np.linalg.norm(b - A.matvec(xg)) <= atol * 1.0001
    assert np.linalg.norm(xg - xr) <= 1e-8 * np.linalg.norm(xr)
