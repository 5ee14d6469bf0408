"""Box-constrained QP on the GPU: MPRGP and multicolour projected Gauss-Seidel against the
oracle (same algorithms restated on the CPU); active sets compared bit-exactly."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def obstacle(N, scaled):
    h = 1.0 / (N + 1)
    return P.obstacle_qp(N, seed=3, rhs=-5 * h * h if scaled else -1.0)


def active(x, lb):
    return x == lb


@pytest.mark.parametrize("N,scaled", [(64, True), (128, False)])
def test_mprgp_matches_oracle(ctx, oracle, N, scaled):
    A, b, lb, ub = obstacle(N, scaled)
    Am = oracle.Matrix(A)
    xo, so = oracle.mprgp_solve(Am, b, lb, ub, atol=1e-10, rtol=1e-14, max_it=5000)
    s = U.MPRGP(ctx, atol=1e-10, rtol=1e-14, max_it=5000)
    vlb, vub = U.Vector(ctx, lb), U.Vector(ctx, ub)
    s.set_box_constraints(vlb, vub)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = s.solution_status()
    xg = x.numpy()
    assert st["converged"] and so["converged"]
    np.testing.assert_allclose(s.get("lambda_max"), so["lambda_max"], rtol=1e-10)
    assert np.array_equal(active(xg, lb), active(xo, lb))
    assert np.linalg.norm(xg - xo) <= 1e-8 * np.linalg.norm(xo)
    assert oracle.projected_gradient_norm(Am, b, lb, ub, xg) <= 1e-9
    assert abs(st["iterates"] - so["iterates"]) <= max(2, 0.05 * so["iterates"])


def test_mprgp_unbounded_is_cg_like(ctx, oracle):
    A, b = P.poisson2d_cg(24, 2)
    s = U.MPRGP(ctx, atol=1e-10, rtol=1e-14, max_it=2000)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    assert np.linalg.norm(A.matvec(x.numpy()) - b) <= 1e-9


def test_pgs_colouring_is_red_black(ctx, oracle):
    A, b, lb, ub = obstacle(40, True)
    s = U.ProjectedGaussSeidel(ctx)
    s.update(U.SparseMatrix(ctx, A))
    col, nc = s.colouring()
    ocol, onc = oracle.colouring(oracle.Matrix(A))
    assert nc == onc == 2
    np.testing.assert_array_equal(col, ocol)
    i = np.arange(A.nrows)
    np.testing.assert_array_equal(col, ((i % 40) + (i // 40)) % 2)


def test_pgs_colouring_general_graph(ctx, oracle):
    A = P.lognormal_diffusion_3d(12, 1)[0]  # 7-point: 2 colours
    L = P.CSR.from_scipy(P.interpolation_3d(8).to_scipy() @ P.interpolation_3d(8).to_scipy().T)  # denser graph
    for M in (A, L):
        s = U.ProjectedGaussSeidel(ctx)
        s.update(U.SparseMatrix(ctx, M))
        col, nc = s.colouring()
        ocol, onc = oracle.colouring(oracle.Matrix(M))
        assert nc == onc
        np.testing.assert_array_equal(col, ocol)


def test_pgs_multicolour_matches_oracle(ctx, oracle):
    A, b, lb, ub = obstacle(48, True)
    Am = oracle.Matrix(A)
    col, nc = oracle.colouring(Am)
    xo, so = oracle.pgs_solve(Am, b, lb, ub, stol=1e-10, max_it=20000, colour=col)
    s = U.ProjectedGaussSeidel(ctx, stol=1e-10, max_it=20000)
    s.set_box_constraints(U.Vector(ctx, lb), U.Vector(ctx, ub))
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = s.solution_status()
    xg = x.numpy()
    assert st["converged"]
    assert abs(st["iterates"] - so["iterates"]) <= 1
    assert np.array_equal(active(xg, lb), active(xo, lb))
    assert np.linalg.norm(xg - xo) <= 1e-7 * np.linalg.norm(xo)


def test_pgs_and_mprgp_agree_on_the_active_set(ctx, oracle):
    A, b, lb, ub = obstacle(48, True)
    Am = oracle.Matrix(A)
    xm, _ = oracle.mprgp_solve(Am, b, lb, ub, atol=1e-11, rtol=1e-14, max_it=5000)
    s = U.ProjectedGaussSeidel(ctx, atol=1e-9, max_it=200000, projected_gradient_stop=1)
    s.set_box_constraints(U.Vector(ctx, lb), U.Vector(ctx, ub))
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xg = x.numpy()
    assert s.solution_status()["converged"]
    assert oracle.projected_gradient_norm(Am, b, lb, ub, xg) <= 1e-9
    # same contact set away from the free boundary's rounding band
    assert (np.abs(xg - lb) < 1e-12).sum() == pytest.approx((np.abs(xm - lb) < 1e-12).sum(), abs=2)


def test_semismooth_newton_matches_oracle(ctx, oracle):
    """SemismoothNewton (utopia_SemismoothNewton_impl.hpp:74-207) through the C ABI on the scaled
    obstacle QP (128^2): same Newton iterations, same final active set and the same minimiser as
    the oracle's restatement, and the MPRGP minimiser."""
    N = 128
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    s = U.SemismoothNewton(ctx, stol=1e-13, max_it=100)
    lbv = U.Vector(ctx, lb)
    s.set_box_constraints(lbv, None)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = s.solution_status()
    xg = x.numpy()
    Am = oracle.Matrix(A)
    xr, ost = oracle.ssn_solve(Am, b, lb=lb, stol=1e-13, max_it=100)
    assert st["converged"] and ost["converged"]
    assert st["iterates"] == ost["iterates"]
    np.testing.assert_array_equal(xg <= lb + 1e-12, xr <= lb + 1e-12)
    assert np.linalg.norm(xg - xr) <= 1e-9 * np.linalg.norm(xr)
    xm, _ = oracle.mprgp_solve(Am, b, lb, ub, atol=1e-12, max_it=50000)
    assert np.linalg.norm(xg - xm) <= 1e-6 * np.linalg.norm(xm)


def test_active_set_compaction_matches_the_predicates(ctx):
    """ugpu_active_set_compact against numpy on the MPRGP predicates, ties at 1e-14 included,
    with and without an upper bound."""
    rng = np.random.default_rng(5)
    n = 1_000_003
    lb = rng.uniform(-1, 0, n)
    ub = lb + rng.uniform(0.5, 1.0, n)
    x = lb + rng.uniform(0, 1, n) * (ub - lb)
    k = rng.integers(0, n, 200_000)
    x[k[:100_000]] = lb[k[:100_000]]                      # on the lower bound
    x[k[100_000:150_000]] = lb[k[100_000:150_000]] + 5e-15  # inside the chop tolerance
    x[k[150_000:]] = ub[k[150_000:]]                      # on the upper bound
    vx, vl, vu = U.Vector(ctx, x), U.Vector(ctx, lb), U.Vector(ctx, ub)
    act = (np.abs(lb - x) < 1e-14) | (np.abs(ub - x) < 1e-14)
    free = (lb < x) & (x < ub)
    np.testing.assert_array_equal(U.active_set(vx, vl, vu, U.SET_ACTIVE), np.flatnonzero(act))
    np.testing.assert_array_equal(U.active_set(vx, vl, vu, U.SET_FREE), np.flatnonzero(free))
    np.testing.assert_array_equal(U.active_set(vx, vl, None, U.SET_ACTIVE), np.flatnonzero(np.abs(lb - x) < 1e-14))
    np.testing.assert_array_equal(U.active_set(vx, vl, None, U.SET_FREE), np.flatnonzero(lb < x))


def test_mprgp_active_set_by_compaction(ctx, oracle):
    """The MPRGP solution's active set, compacted on the device, equals the oracle's."""
    A, b, lb, ub = obstacle(128, False)
    xo, _ = oracle.mprgp_solve(oracle.Matrix(A), b, lb, ub, atol=1e-10, rtol=1e-14, max_it=5000)
    s = U.MPRGP(ctx, atol=1e-10, rtol=1e-14, max_it=5000)
    vlb, vub = U.Vector(ctx, lb), U.Vector(ctx, ub)
    s.set_box_constraints(vlb, vub)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    got = U.active_set(x, vlb, vub, U.SET_ACTIVE)
    np.testing.assert_array_equal(got, np.flatnonzero((np.abs(lb - xo) < 1e-14) | (np.abs(ub - xo) < 1e-14)))


def test_vector_reductions_and_transforms(ctx):
    rng = np.random.default_rng(6)
    v = rng.standard_normal(300_001)
    dv = U.Vector(ctx, v)
    np.testing.assert_allclose(U.reduce(dv, U.RED_SUM), v.sum(), rtol=1e-12)
    assert U.reduce(dv, U.RED_MIN) == v.min() and U.reduce(dv, U.RED_MAX) == v.max()
    np.testing.assert_allclose(U.reduce(dv, U.RED_ASUM), np.abs(v).sum(), rtol=1e-12)
    assert U.reduce(dv, U.RED_AMAX) == np.abs(v).max()
    lib = ctx.lib
    for op, param, f in ((6, 0.0, np.abs), (7, 0.0, np.negative), (10, 2.5, lambda a: a + 2.5),
                         (11, -3.0, lambda a: a * -3.0), (1, 0.0, lambda a: a * a)):
        w = U.Vector(ctx, v)
        assert lib.ugpu_vec_transform(w.h, op, param) == 0
        np.testing.assert_allclose(w.numpy(), f(v), rtol=1e-15)


def test_mprgp_graph_and_eager_are_bitwise_equal(ctx, oracle):
    """The graph form (the iteration under a WHILE node, the expansion tail under an IF node set on
    the device) and the eager form (every kernel launched, the tail gated inside its kernels) give
    the same iterates bit for bit on a problem with expansion steps; both match the oracle's
    active set."""
    N = 96
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-10.0 * h * h)
    atol = 1e-9 * h * h
    out = {}
    for graphs in (1, 0):
        s = U.MPRGP(ctx, atol=atol, rtol=1e-30, max_it=100000, use_graphs=graphs)
        s.set_box_constraints(U.Vector(ctx, lb), U.Vector(ctx, ub))
        x = U.Vector(ctx, n=A.nrows)
        s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
        out[graphs] = (x.numpy(), s.solution_status())
    (xg, sg), (xe, se) = out[1], out[0]
    assert sg["converged"] and se["converged"]
    assert sg["iterates"] == se["iterates"]
    assert np.array_equal(xg, xe)
    xo, so = oracle.mprgp_solve(oracle.Matrix(A), b, lb, ub, atol=atol, rtol=1e-30, max_it=100000)
    assert np.array_equal(xg == lb, xo == lb)


def _penalty_gpu(ctx, A, b, ub=None, lb=None, selection=None, T=None, O=None, S=None, x0=None, solver=None, **prm):
    s = solver or U.ShiftedPenaltyQPSolver(ctx, **prm)
    keep = [U.Vector(ctx, v) if v is not None else None for v in (lb, ub, selection)]
    s.set_box_constraints(keep[0], keep[1])
    if selection is not None:
        s.set_selection(keep[2])
    mats = [U.SparseMatrix(ctx, M) if M is not None else None for M in (T, O, S)]
    if T is not None:
        s.set_transform(mats[0], mats[1])
    if S is not None:
        s.set_scaling_matrix(mats[2])
    x = U.Vector(ctx, x0) if x0 is not None else U.Vector(ctx, n=A.nrows)
    Ad = U.SparseMatrix(ctx, A)
    s.solve(Ad, U.Vector(ctx, b), x)
    return x.numpy(), s.solution_status(), s, (keep, mats, Ad)


def test_shifted_penalty_reference_test_problem(ctx, oracle):
    """ShiftedPenaltyQPSolver on the reference's own test problem (utopia_QPSolverTest.cpp:407-424:
    1D Laplacian, n = 20, upper bound 30, max_it 40 n) through the C ABI: the oracle's iterations
    and reason, x to 1e-12 and below the bound up to the penalty's residual violation."""
    A, b, ub = P.qp_test_problem_1d(20)
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, ub=ub, max_it=800)
    xg, st, _, _ = _penalty_gpu(ctx, A, b, ub=ub, max_it=800)
    assert st["converged"] and so["converged"]
    assert st["iterates"] == so["iterates"] and st["reason"] == so["reason"]
    assert np.linalg.norm(xg - xo) <= 1e-12 * np.linalg.norm(xo)
    assert xg.max() <= 30.0 + 1e-6 and xg.max() >= 30.0 - 1e-6


@pytest.mark.parametrize("variant", ["plain", "selection_scaling", "transformation"])
def test_shifted_penalty_matches_oracle(ctx, oracle, variant):
    """128^2 Laplacian with an upper bound (contact under a load), plain, with a 0/1 selection and a
    diagonal scaling matrix, and with the qp_solve app's transformation (T block rotations, O block
    reflections: the reference maps the Hessian by T^T O^T D O T and directions by T^T O, which agree
    for a symmetric O):
    same iterations and reason as the oracle (pinned bit for bit to the reference's solver), x to
    1e-9, and in the plain case the MPRGP minimiser to 1e-6."""
    N = 128
    h = 1.0 / (N + 1)
    A, b, _, _ = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    b = -b
    n = A.nrows
    cap = np.full(n, 0.02)
    rng = np.random.default_rng(1)
    kw = dict(ub=cap)
    if variant == "selection_scaling":
        kw["selection"] = (rng.uniform(size=n) < 0.8).astype(float)
        import scipy.sparse as sp
        kw["S"] = P.CSR.from_scipy(sp.diags(rng.uniform(0.5, 2.0, n)).tocsr())
    if variant == "transformation":
        kw["T"], kw["O"] = P.block_rotation(n, 5), P.block_rotation(n, 7, reflection=True)
    okw = {k: (oracle.Matrix(v) if isinstance(v, P.CSR) else v) for k, v in kw.items()}
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, max_it=300, **okw)
    xg, st, _, _ = _penalty_gpu(ctx, A, b, max_it=300, **kw)
    assert so["converged"] and st["converged"]
    assert st["iterates"] == so["iterates"] and st["reason"] == so["reason"]
    assert np.linalg.norm(xg - xo) <= 1e-9 * np.linalg.norm(xo)
    w = xg
    if variant == "transformation":
        w = kw["O"].to_scipy().T @ (kw["T"].to_scipy() @ xg)
    sel = kw["selection"] != 0 if "selection" in kw else np.ones(n, bool)
    assert (w - cap)[sel].max() <= 1e-12 and (w >= cap - 1e-9).sum() > 100  # a real contact set
    if variant == "plain":
        Am = oracle.Matrix(A)
        xm, sm = oracle.mprgp_solve(Am, b, np.full(n, -np.finfo(float).max), cap, atol=1e-12, max_it=50000)
        assert sm["converged"]
        assert np.linalg.norm(xg - xm) <= 1e-6 * np.linalg.norm(xm)


def test_shifted_penalty_lower_bound_is_inert(ctx, oracle):
    """As in the reference, a lower bound alone is not enforced (the missing upper bound is filled
    with the largest double and update_shift_aux takes its upper-bound branch): the solve returns
    the unconstrained minimiser, as the oracle does."""
    N = 64
    h = 1.0 / (N + 1)
    A, b, lb, _ = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, lb=lb, max_it=50)
    xg, st, _, _ = _penalty_gpu(ctx, A, b, lb=lb, max_it=50)
    assert st["iterates"] == so["iterates"] == 2
    assert np.linalg.norm(xg - xo) <= 1e-10 * np.linalg.norm(xo)
    assert (xg < lb).any()


def test_shifted_penalty_warm_shift_and_linear_solver_slot(ctx, oracle):
    """zero_shift_on_reset 0: the second solve by the same solver starts from the first one's
    shift (fewer iterations, the oracle's count); a caller-set inner solver (CG + Jacobi at a
    tighter tolerance) takes the place of the default one."""
    N = 64
    h = 1.0 / (N + 1)
    A, b, _, _ = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    b = -b
    n = A.nrows
    cap = np.full(n, 0.02)
    T, O = P.block_rotation(n, 5), P.block_rotation(n, 7, reflection=True)
    To, Oo = oracle.Matrix(T), oracle.Matrix(O)
    x1, s1, shift = oracle.penalty_solve(oracle.Matrix(A), b, ub=cap, T=To, O=Oo, max_it=200)
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, x0=x1, ub=cap, T=To, O=Oo, shift=shift, max_it=200)
    s = U.ShiftedPenaltyQPSolver(ctx, max_it=200, zero_shift_on_reset=0)
    xg1, st1, s, keep = _penalty_gpu(ctx, A, b, ub=cap, T=T, O=O, solver=s)
    assert st1["iterates"] == s1["iterates"]
    xv = U.Vector(ctx, xg1)
    s.apply(U.Vector(ctx, b), xv)
    st2 = s.solution_status()
    assert st2["iterates"] == so["iterates"] < s1["iterates"]
    assert np.linalg.norm(xv.numpy() - xo) <= 1e-9 * np.linalg.norm(xo)
    # the inner-solver slot
    cg = U.ConjugateGradient(ctx, atol=1e-14, max_it=20000)
    cg.set_preconditioner(U.InvDiagPreconditioner(ctx))
    s2 = U.ShiftedPenaltyQPSolver(ctx, max_it=200)
    s2.set_linear_solver(cg)
    xg, st, _, _ = _penalty_gpu(ctx, A, b, ub=cap, solver=s2)
    xp, sp_, _ = oracle.penalty_solve(oracle.Matrix(A), b, ub=cap, max_it=200)
    assert st["converged"]
    assert np.linalg.norm(xg - xp) <= 1e-8 * np.linalg.norm(xp)


def test_qp_solve_shifted_penalty_app(ctx, oracle, tmp_path):
    """The reference's qp_solve app (QPSolveApp::solve_with_shifted_penalty, utopia_qp_solve.cpp:
    61-107) on files: A, T, O, rhs, upper_bound, is_contact; the constraint acts on O^T (T x).  The
    written x is the oracle's shifted-penalty solution with the same transformation."""
    from utopia_gb300 import qp_solve

    N = 64
    h = 1.0 / (N + 1)
    A, b, _, _ = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    b = -b
    n = A.nrows
    cap = np.full(n, 0.02)
    T, O = P.block_rotation(n, 5), P.block_rotation(n, 7, reflection=True)
    for name, m in (("A", A), ("T", T), ("O", O)):
        U.SparseMatrix(ctx, m).write_petsc(str(tmp_path / name))
    for name, v in (("rhs", b), ("upper_bound", cap), ("is_contact", np.ones(n))):
        U.Vector(ctx, v).write_petsc(str(tmp_path / name))
    out = qp_solve.main(["--dir", str(tmp_path), "--solver", "shifted_penalty", "--max_it", "200",
                         "--out", str(tmp_path / "out.bin")])
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, ub=cap, T=oracle.Matrix(T), O=oracle.Matrix(O),
                                     max_it=200)
    assert out["converged"] and so["converged"] and out["iterations"] == so["iterates"]
    assert out["violation"] <= 1e-12
    x = U.read_petsc_vector(ctx, str(tmp_path / "out.bin")).numpy()
    assert np.linalg.norm(x - xo) <= 1e-9 * np.linalg.norm(xo)
