"""The restated oracle (oracle/oracle.cpp) against the reference's own solver templates,
compiled from the reference checkout over a CPU CSR backend (oracle/ref/, built into
oracle/_ref/ by oracle.ref.build_ref).  Both run on the same seeded inputs; they agree bit
for bit: iteration counts, convergence reasons, solutions, Galerkin structures and values,
stand-alone multigrid iterates, MPRGP and projected Gauss-Seidel active sets.

CPU only.  Skipped where the reference checkout is not present.
"""
import numpy as np
import pytest

from utopia_gb300 import problems as P

ref = pytest.importorskip("oracle.ref")
if not ref.reference_available():
    pytest.skip("the reference checkout is not present", allow_module_level=True)


@pytest.fixture(scope="module")
def R():
    ref.build_ref()
    return ref


def same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b))


def test_cg_invdiag_poisson2d_256(oracle, R):
    """ConjugateGradient + InvDiagPreconditioner on the 256^2 Poisson problem, atol 1e-8 ||b||."""
    A, b = P.poisson2d_cg(256, 0)
    atol = 1e-8 * np.linalg.norm(b)
    xo, so = oracle.cg_solve(oracle.Matrix(A), b, atol=atol)
    xr, sr = R.cg_solve(R.Matrix(A), b, atol=atol)
    assert so["iterates"] == sr["iterates"] and so["reason"] == sr["reason"] == 2
    assert same(xo, xr)


def test_cg_unpreconditioned(oracle, R):
    A, b = P.poisson2d_cg(48, 4)
    xo, so = oracle.cg_solve(oracle.Matrix(A), b, precond="none", atol=1e-9)
    xr, sr = R.cg_solve(R.Matrix(A), b, precond="none", atol=1e-9)
    assert so["iterates"] == sr["iterates"]
    assert same(xo, xr)


CASES = {
    "poisson32_chebyshev": (lambda: P.poisson3d_mg(32, 3, seed=1), "chebyshev", 3),
    "poisson64_chebyshev_4levels": (lambda: P.poisson3d_mg(64, 4, seed=1), "chebyshev", 3),
    "lognormal32_jacobi": (lambda: P.lognormal_mg(32, 3, seed=2), "jacobi", 2),
    "lognormal32_point_jacobi": (lambda: P.lognormal_mg(32, 3, seed=2), "point_jacobi", 2),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_mg_pcg(oracle, R, case):
    """Multigrid-preconditioned CG: Galerkin operators (structure and values) of every level,
    PowerMethod eigen-bounds (through the iterates), iterations and x, bit for bit."""
    make, smoother, nu = CASES[case]
    A, Ps, b = make()
    atol = 1e-10 * np.linalg.norm(b)
    Ao, Ar = oracle.Matrix(A), R.Matrix(A)
    mo = oracle.Multigrid(Ao, Ps, smoother=smoother, pre=nu, post=nu)
    mr = R.Multigrid(Ar, Ps, smoother=smoother, pre=nu, post=nu)
    assert mo.n_levels == mr.n_levels
    for lev in range(mo.n_levels):
        for u, v in zip(mo.level_matrix(lev).arrays(), mr.level_matrix_arrays(lev)):
            assert same(u, v), f"level {lev}"
    xo, so = oracle.cg_solve(Ao, b, precond="mg", mg=mo, atol=atol)
    xr, sr = R.cg_solve(Ar, b, precond="mg", mg=mr, atol=atol)
    assert so["iterates"] == sr["iterates"]
    assert same(xo, xr)
    # Multigrid::apply as a stand-alone solver: the iterates after 1..3 cycles
    for k in (1, 2, 3):
        xo, so = mo.solve(b, atol=0.0, rtol=0.0, max_it=k)
        xr, sr = mr.solve(b, atol=0.0, rtol=0.0, max_it=k)
        assert so["iterates"] == sr["iterates"] == k
        assert so["gradient_norm"] == sr["gradient_norm"]
        assert same(xo, xr)


def test_mg_pcg_reference_fixture_with_masks(oracle, R, laplace_hierarchy):
    """petsc_cg_mg's 4-level fixture (Dirichlet identity rows, so non-trivial multilevel
    masks), Chebyshev smoothing, atol 1e-10."""
    A, Is, rhs = laplace_hierarchy
    Ao, Ar = oracle.Matrix(A), R.Matrix(A)
    mo = oracle.Multigrid(Ao, Is, smoother="chebyshev", pre=3, post=3)
    mr = R.Multigrid(Ar, Is, smoother="chebyshev", pre=3, post=3)
    xo, so = oracle.cg_solve(Ao, rhs, precond="mg", mg=mo, atol=1e-10)
    xr, sr = R.cg_solve(Ar, rhs, precond="mg", mg=mr, atol=1e-10)
    assert so["iterates"] == sr["iterates"]
    assert same(xo, xr)


@pytest.mark.parametrize("N,scale", [(1024, None), (64, 5.0), (128, 20.0)])
def test_mprgp(oracle, R, N, scale):
    """MPRGP on the obstacle problem: the 1024^2 case as specified (b = -1) and two scaled
    right-hand sides with a free boundary; iterations, reason, active set and x bit for bit."""
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-1.0 if scale is None else -scale * h * h)
    atol = 1e-8 if scale is None else 1e-8 * h * h
    xo, so = oracle.mprgp_solve(oracle.Matrix(A), b, lb, ub, atol=atol, rtol=1e-30, max_it=100000)
    xr, sr = R.mprgp_solve(R.Matrix(A), b, lb, ub, atol=atol, rtol=1e-30, max_it=100000)
    assert so["iterates"] == sr["iterates"] and so["reason"] == sr["reason"]
    assert same(xo == lb, xr == lb)
    assert same(xo, xr)


def test_projected_gauss_seidel_lexicographic(oracle, R):
    """ProjectedGaussSeidel (lexicographic, 3 symmetric local sweeps, stop on ||x - x_old||)."""
    N = 64
    h = 1.0 / (N + 1)
    A, b, lb, ub = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    xo, so = oracle.pgs_solve(oracle.Matrix(A), b, lb, ub, stol=1e-11, max_it=50000)
    xr, sr = R.pgs_solve(R.Matrix(A), b, lb, ub, stol=1e-11, max_it=50000)
    assert so["iterates"] == sr["iterates"] and so["reason"] == sr["reason"]
    assert same(xo == lb, xr == lb)
    assert same(xo, xr)


def _penalty_cases():
    N = 32
    h = 1.0 / (N + 1)
    A, b, lb, _ = P.obstacle_qp(N, seed=3, rhs=-5 * h * h)
    n = A.nrows
    rng = np.random.default_rng(1)
    sel = (rng.uniform(size=n) < 0.8).astype(float)
    S = P.CSR.from_scipy(__import__("scipy.sparse", fromlist=["diags"]).diags(rng.uniform(0.5, 2.0, n)).tocsr())
    cap = np.full(n, 0.02)
    T, O = P.block_rotation(n, 5), P.block_rotation(n, 7, reflection=True)
    A1, b1, ub1 = P.qp_test_problem_1d(20)
    return {
        "qp_test_problem_1d": (A1, b1, dict(ub=ub1, max_it=800)),
        "upper_bound": (A, -b, dict(ub=cap, max_it=200)),
        "lower_bound_is_inert": (A, b, dict(lb=lb, max_it=200)),
        "selection_and_scaling": (A, -b, dict(ub=cap, selection=sel, S=S, max_it=200)),
        "transformation": (A, -b, dict(ub=cap, T=T, O=O, max_it=200)),
        "growing_penalty": (A, -b, dict(ub=cap, T=T, O=O, penalty_parameter=1e2, penalty_parameter_max=1e6,
                                        max_it=200)),
    }


@pytest.mark.parametrize("case", ["qp_test_problem_1d", "upper_bound", "lower_bound_is_inert",
                                  "selection_and_scaling", "transformation", "growing_penalty"])
def test_shifted_penalty(oracle, R, case):
    """ShiftedPenaltyQPSolver + ShiftedPenalty (with the qp_solve app's transformation, a
    selection and a scaling matrix): iterations, reason and x bit for bit.  The first case is the
    reference's own test problem (utopia_QPSolverTest.cpp:407-424, QPSolverTestProblem)."""
    A, b, kw = _penalty_cases()[case]

    def mats(M):
        return {k: (M(v) if isinstance(v, P.CSR) else v) for k, v in kw.items()}

    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, **mats(oracle.Matrix))
    xr, sr = R.penalty_solve(R.Matrix(A), b, **mats(R.Matrix))
    assert so["iterates"] == sr["iterates"] and so["reason"] == sr["reason"] and so["converged"]
    assert same(xo, xr)
    w = xo if "T" not in kw else kw["O"].to_scipy().T @ (kw["T"].to_scipy() @ xo)
    if "ub" in kw:  # the constraint holds where it is selected
        sel = kw["selection"] != 0 if "selection" in kw else np.ones(w.size, bool)
        assert (w - kw["ub"])[sel].max() <= 1e-10


def test_shifted_penalty_keeps_its_shift(oracle, R):
    """zero_shift_on_reset false: a second solve by the same solver object starts from the
    previous solve's shift (ShiftedPenalty::reset, utopia_ShiftedPenalty.hpp:552-566)."""
    A, b, kw = _penalty_cases()["transformation"]
    T, O = oracle.Matrix(kw["T"]), oracle.Matrix(kw["O"])
    x1, s1, shift = oracle.penalty_solve(oracle.Matrix(A), b, ub=kw["ub"], T=T, O=O, max_it=200)
    xo, so, _ = oracle.penalty_solve(oracle.Matrix(A), b, x0=x1, ub=kw["ub"], T=T, O=O, shift=shift, max_it=200)
    xr, sr = R.penalty_solve(R.Matrix(A), b, ub=kw["ub"], T=R.Matrix(kw["T"]), O=R.Matrix(kw["O"]),
                             zero_shift_on_reset=False, n_solves=2, max_it=200)
    assert so["iterates"] == sr["iterates"] < s1["iterates"]
    assert same(xo, xr)
