"""MonotoneMultigrid through the C ABI against the oracle's restatement of
utopia_MonotoneMultigrid.hpp:135-319: the reference's 1D obstacle case
(utopia/tests/utopia_QPSolverTest.cpp:715-771), a 2D obstacle problem with the multigrid and the
dense coarse solve below the truncated level, and more than one coarse cycle per step."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def run_gpu(ctx, A, b, lb, ub, Ps, **kw):
    s = U.MonotoneMultigrid(ctx, **kw)
    s.set_transfer_operators(Ps)
    lbv = U.Vector(ctx, lb) if lb is not None else None
    ubv = U.Vector(ctx, ub) if ub is not None else None
    s.set_box_constraints(lbv, ubv)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    return s, x.numpy(), s.solution_status()


def test_monotone_mg_reference_1d_case(ctx, oracle):
    H, g, lb, ub, Ps = P.poisson1d_obstacle_multilevel()
    Am = oracle.Matrix(H)
    colour = oracle.colouring(Am)[0]
    kw = dict(pre_smoothing_steps=5, post_smoothing_steps=5, max_it=40, active_set_tol=1e-15)
    s, x, st = run_gpu(ctx, H, g, lb, ub, Ps, **kw)
    xr, ost, act, AH = oracle.monotone_mg_solve(Am, g, lb, ub, Ps, colour=colour, pre=5, post=5, max_it=40,
                                                active_tol=1e-15)
    assert st["converged"] and ost["converged"]
    assert abs(st["iterates"] - ost["iterates"]) <= 1
    np.testing.assert_array_equal(s.active_set(), act)
    assert s.get("n_active") == act.sum() and s.get("galerkin_assemblies") >= 2
    assert np.abs(x - xr).max() < 1e-10
    # the minimiser: the semismooth Newton restatement's
    xs, _ = oracle.ssn_solve(Am, g, lb, ub, stol=1e-14)
    assert np.abs(x - xs).max() < 1e-9
    # levels: the fine operator on top, the truncated Galerkin operator below it (same
    # structure as the oracle's, fixed identity rows for fully active coarse dofs)
    assert s.n_levels() == 6
    G = s.level_matrix(4)
    rp, ci, v = G.csr()
    orp, oci, ov = AH.arrays()
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    np.testing.assert_allclose(v, ov, rtol=1e-12, atol=1e-12 * np.abs(ov).max())


@pytest.mark.parametrize("levels,csi", [(4, 1), (4, 2), (2, 1)])
def test_monotone_mg_obstacle_2d(ctx, oracle, levels, csi):
    N = 64
    h = 1.0 / (N + 1)
    A, b, lb, _ = P.obstacle_qp(N, seed=3, rhs=-20 * h * h)
    Ps = P.hierarchy_2d(N, levels)
    Am = oracle.Matrix(A)
    colour = oracle.colouring(Am)[0]
    atol = 1e-10 * h * h
    s, x, st = run_gpu(ctx, A, b, lb, None, Ps, max_it=200, atol=atol, coarse_space_it=csi)
    xr, ost, act, _ = oracle.monotone_mg_solve(Am, b, lb, None, Ps, colour=colour, max_it=200, atol=atol,
                                               coarse_space_it=csi)
    assert st["converged"] and ost["converged"]
    assert abs(st["iterates"] - ost["iterates"]) <= 1
    assert s.n_levels() == levels
    np.testing.assert_array_equal(s.active_set(), act)
    assert np.abs(x - xr).max() < 1e-12
    assert np.all(x >= lb - 1e-14)
    xs, _ = oracle.ssn_solve(Am, b, lb, None, stol=1e-14)
    assert np.abs(x - xs).max() < 1e-10


def test_monotone_mg_errors(ctx):
    A = P.laplacian_2d(8)
    s = U.MonotoneMultigrid(ctx)
    with pytest.raises(U.UgpuError):  # no transfer operators
        s.update(U.SparseMatrix(ctx, A))
    with pytest.raises(U.UgpuError):  # interpolations that do not chain coarse -> fine
        s.set_transfer_operators(P.hierarchy_2d(8, 3)[::-1])
    with pytest.raises(U.UgpuError):  # the fine transfer does not match the operator
        s.set_transfer_operators(P.hierarchy_2d(16, 2))
        s.update(U.SparseMatrix(ctx, A))
