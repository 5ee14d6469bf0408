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


def contact_rotation(n: int, pairs, seed: int) -> P.CSR:
    """A symmetric orthogonal contact transformation: 2x2 reflections [[c, s], [s, -c]] on the dof
    pairs (2k, 2k+1) for k in `pairs`, the identity elsewhere (Rot = Rot^T = Rot^-1)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    R = sp.lil_matrix((n, n))
    for i in range(n):
        R[i, i] = 1.0
    for k in pairs:
        t = rng.uniform(0, np.pi)
        c, s = np.cos(t), np.sin(t)
        i, j = 2 * k, 2 * k + 1
        R[i, i], R[i, j], R[j, i], R[j, j] = c, s, s, -c
    return P.CSR.from_scipy(R.tocsr())


@pytest.mark.parametrize("solver", ["monotone_mg", "semismooth_newton"])
def test_qp_solve_app_with_contact_rotation(ctx, oracle, tmp_path, solver):
    """qp_solve (MGQPSolveApp without QR, utopia_qp_solve.cpp:90-330) on files written in the
    original coordinates of a rotated 2D obstacle problem: the app rotates A, rhs, x and the fine
    interpolation, solves in the rotated coordinates and writes x = Rot x'; the result is the
    oracle's monotone multigrid solution of the same rotated system, rotated back."""
    from utopia_gb300 import qp_solve

    N = 64
    h = 1.0 / (N + 1)
    A1, b1, lb, _ = P.obstacle_qp(N, seed=3, rhs=-20 * h * h)
    ub = np.full(A1.nrows, np.finfo(np.float64).max)
    Ps = P.hierarchy_2d(N, 4)
    n = A1.nrows
    Rot = contact_rotation(n, range(0, n // 2, 3), 7)
    Rs = Rot.to_scipy()
    A = P.CSR.from_scipy(Rs @ A1.to_scipy() @ Rs)
    rhs = Rs @ b1
    I_last = P.CSR.from_scipy(Rs @ Ps[-1].to_scipy())
    for name, m in (("A", A), ("Rot", Rot), ("I1", Ps[0]), ("I2", Ps[1]), ("I3", I_last)):
        U.SparseMatrix(ctx, m).write_petsc(str(tmp_path / name))
    for name, v in (("rhs", rhs), ("x", np.zeros(n)), ("lb", lb), ("ub", ub)):
        U.Vector(ctx, v).write_petsc(str(tmp_path / name))
    atol = 1e-10 * h * h
    out = qp_solve.main(["--dir", str(tmp_path), "--n_interpolators", "3", "--max_it", "200", "--atol", str(atol),
                         "--stol", "1e-14", "--solver", solver, "--out", str(tmp_path / "x_out")])
    assert out["converged"] and out["bound_violation"] == 0.0
    x = U.read_petsc_vector(ctx, str(tmp_path / "x_out")).numpy()
    Rm = oracle.Matrix(Rot)
    Ar = Rm.matmul(oracle.Matrix(A)).matmul(Rm)
    Ir = Rm.matmul(oracle.Matrix(I_last))
    xr, ost, act, _ = oracle.monotone_mg_solve(Ar, Rs @ rhs, lb, ub, [Ps[0], Ps[1], Ir],
                                               colour=oracle.colouring(Ar)[0], max_it=200, atol=atol, stol=1e-14)
    assert ost["converged"]
    if solver == "monotone_mg":
        assert abs(out["iterations"] - ost["iterates"]) <= 1
        assert out["n_active"] == act.sum()
    xo = Rs @ xr
    assert np.linalg.norm(x - xo) <= 1e-9 * np.linalg.norm(xo)
