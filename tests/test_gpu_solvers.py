"""GPU solver parity against the oracle (iteration counts, Galerkin structure,
eigen-bounds, solutions), through the C ABI."""
import hashlib
import json
import os

import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def cg(ctx, prec=None, **kw):
    s = U.ConjugateGradient(ctx, **kw)
    if prec is not None:
        s.set_preconditioner(prec)
    return s


@pytest.mark.parametrize("graphs", [1, 0])
def test_cg_jacobi_poisson2d_256(ctx, oracle, graphs):
    """Plain FP64 CG + InvDiag on the 2D 5-point Laplacian 256^2, b ~ U[-1,1] (seed 0),
    x0 = 0, atol = 1e-8 ||b|| (CG stops only on atol, utopia_ConjugateGradient_impl.hpp:258)."""
    A, b = P.poisson2d_cg(256, 0)
    atol = 1e-8 * np.linalg.norm(b)
    xo, so = oracle.cg_solve(oracle.Matrix(A), b, atol=atol)
    s = cg(ctx, U.InvDiagPreconditioner(ctx), atol=atol, use_graphs=graphs)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = s.solution_status()
    assert abs(st["iterates"] - so["iterates"]) <= 1
    assert st["reason"] == 2 and st["gradient_norm"] <= atol
    xg = x.numpy()
    assert np.linalg.norm(b - A.matvec(xg)) <= atol * 1.001
    assert rel(xg, xo) <= 1e-6


def test_cg_graph_and_eager_are_bitwise_equal(ctx):
    A, b = P.poisson2d_cg(64, 0)
    outs = []
    for graphs in (1, 0, 1):
        s = cg(ctx, U.InvDiagPreconditioner(ctx), atol=1e-9, use_graphs=graphs)
        x = U.Vector(ctx, n=A.nrows)
        s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
        outs.append((x.numpy(), s.solution_status()["iterates"]))
    for xo, it in outs[1:]:
        np.testing.assert_array_equal(xo, outs[0][0])
        assert it == outs[0][1]


def test_cg_unpreconditioned(ctx, oracle):
    A, b = P.poisson2d_cg(48, 4)
    xo, so = oracle.cg_solve(oracle.Matrix(A), b, precond="none", atol=1e-10)
    s = cg(ctx, None, atol=1e-10)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    assert abs(s.solution_status()["iterates"] - so["iterates"]) <= 1
    assert rel(x.numpy(), xo) <= 1e-8


def test_cg_max_it_and_initial_guess(ctx, oracle):
    A, b = P.poisson2d_cg(32, 1)
    x0 = np.random.default_rng(3).standard_normal(A.nrows)
    xo, so = oracle.cg_solve(oracle.Matrix(A), b, x0=x0, atol=1e-30, max_it=7)
    s = cg(ctx, U.InvDiagPreconditioner(ctx), atol=1e-30, max_it=7)
    x = U.Vector(ctx, x0)
    assert not s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    st = s.solution_status()
    assert st["reason"] == -5 and st["iterates"] == so["iterates"] == 7
    assert rel(x.numpy(), xo) <= 1e-12


def test_cg_zero_rhs_reports_nan_stop(ctx, oracle):
    # b = 0: r = z = p = 0 and alpha = 0/0; the reference breaks out unconverged
    A, b = P.poisson2d_cg(16, 1)
    b[:] = 0
    xo, so = oracle.cg_solve(oracle.Matrix(A), b)
    s = cg(ctx, U.InvDiagPreconditioner(ctx))
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x) == bool(so["converged"])
    assert not np.isnan(x.numpy()).any()


def test_cg_nan_in_rhs_does_not_converge(ctx):
    A, b = P.poisson2d_cg(16, 1)
    b[5] = np.nan
    s = cg(ctx, U.InvDiagPreconditioner(ctx))
    x = U.Vector(ctx, n=A.nrows)
    assert not s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    assert s.solution_status()["reason"] < 0


def _mg(ctx, Ps, **kw):
    mg = U.Multigrid(ctx, **kw)
    mg.set_transfer_operators(Ps)
    return mg


def test_mgpcg_chebyshev_pins(ctx, oracle):
    """MG-PCG (Chebyshev 3+3, dense Cholesky coarse) on 32^3, 3 levels: Galerkin structure
    digests, eigen-bounds and iteration count against the committed pins."""
    pins = json.load(open(os.path.join(GOLDEN, "pins.json")))
    A, Ps, b = P.poisson3d_mg(32, 3, seed=1)
    mg = _mg(ctx, Ps, smoother="chebyshev", pre_smoothing_steps=3, post_smoothing_steps=3)
    s = cg(ctx, mg, atol=1e-10 * np.linalg.norm(b))
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    for l in range(mg.n_levels()):
        rp, ci, _ = mg.level_matrix(l).csr()
        assert hashlib.sha256(rp.tobytes() + ci.tobytes()).hexdigest() == pins["galerkin_poisson3d_32"][f"level{l}"]
    for l in range(1, mg.n_levels()):
        np.testing.assert_allclose(mg.eigs(l), pins["galerkin_poisson3d_32"]["eigs"][l - 1], rtol=1e-9)
    assert abs(s.solution_status()["iterates"] - pins["mgpcg_chebyshev_poisson3d_32"]["iterates"]) <= 1


def test_mgpcg_poisson3d_128_full(ctx, oracle):
    """The 128^3 configuration: 4 levels, trilinear P, R = P^T, Galerkin RAP, Chebyshev 3+3,
    dense FP64 Cholesky on 16^3, atol = 1e-10 ||b||.  RAP structure bit-exact, iteration
    count within 1 and x within 1e-9 relative L2 of the oracle."""
    A, Ps, b = P.poisson3d_mg(128, 4, seed=1)
    atol = 1e-10 * np.linalg.norm(b)
    Am = oracle.Matrix(A)
    omg = oracle.Multigrid(Am, Ps, smoother="chebyshev", pre=3, post=3)
    xo, so = oracle.cg_solve(Am, b, precond="mg", mg=omg, atol=atol)
    mg = _mg(ctx, Ps, smoother="chebyshev")
    s = cg(ctx, mg, atol=atol)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    for l in range(mg.n_levels() - 1):
        rp, ci, v = mg.level_matrix(l).csr()
        orp, oci, ov = omg.level_matrix(l).arrays()
        assert (rp == orp).all() and (ci == oci).all()
        np.testing.assert_allclose(v, ov, rtol=1e-12, atol=1e-14)
    for l in range(1, mg.n_levels()):
        np.testing.assert_allclose(mg.eigs(l), omg.eigs(l), rtol=1e-9)
    assert abs(s.solution_status()["iterates"] - so["iterates"]) <= 1
    assert rel(x.numpy(), xo) <= 1e-9


@pytest.mark.parametrize("smoother,omega", [("jacobi", 1.0), ("jacobi", 0.8), ("point_jacobi", 1.0)])
def test_mgpcg_jacobi_smoothers(ctx, oracle, smoother, omega):
    A, Ps, b = P.lognormal_mg(32, 3, seed=2)
    atol = 1e-10 * np.linalg.norm(b)
    Am = oracle.Matrix(A)
    omg = oracle.Multigrid(Am, Ps, smoother=smoother, pre=2, post=2, omega=omega)
    xo, so = oracle.cg_solve(Am, b, precond="mg", mg=omg, atol=atol)
    mg = _mg(ctx, Ps, smoother=smoother, omega=omega, pre_smoothing_steps=2, post_smoothing_steps=2)
    s = cg(ctx, mg, atol=atol)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    assert abs(s.solution_status()["iterates"] - so["iterates"]) <= 1
    assert rel(x.numpy(), xo) <= 1e-9


def test_reference_fixture_cg_mg_with_masks(ctx, oracle, laplace_hierarchy):
    """petsc_cg_mg on the reference's 4-level fixture (Dirichlet rows -> non-trivial masks,
    fix_semidefinite_operators on): the reference asserts A x ~= rhs to 1e-6."""
    A, Is, rhs = laplace_hierarchy
    mg = _mg(ctx, Is, smoother="jacobi", pre_smoothing_steps=3, post_smoothing_steps=3,
             fix_semidefinite_operators=1, must_generate_masks=1)
    s = cg(ctx, mg, atol=1e-10, rtol=1e-18, stol=1e-18)
    x = U.Vector(ctx, rhs)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, rhs), x)
    assert np.allclose(A.matvec(x.numpy()), rhs, atol=1e-6)
    omg = oracle.Multigrid(oracle.Matrix(A), Is, smoother="jacobi", pre=3, post=3, fix_semidefinite=True)
    xo, so = oracle.cg_solve(oracle.Matrix(A), rhs, x0=rhs, precond="mg", mg=omg, atol=1e-10, rtol=1e-18,
                             stol=1e-18)
    assert abs(s.solution_status()["iterates"] - so["iterates"]) <= 1


def test_reference_fixture_mg_point_jacobi_solver(ctx, laplace_hierarchy):
    """petsc_mg_jacobi: Multigrid with PointJacobi as a stand-alone solver, A x ~= rhs to 1e-6."""
    A, Is, rhs = laplace_hierarchy
    mg = _mg(ctx, Is, smoother="point_jacobi")
    x = U.Vector(ctx, n=A.nrows)
    mg.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, rhs), x)
    assert np.allclose(A.matvec(x.numpy()), rhs, atol=1e-6)


def test_vcycle_matches_oracle(ctx, oracle):
    A, Ps, b = P.lognormal_mg(32, 3, seed=7)
    omg = oracle.Multigrid(oracle.Matrix(A), Ps, smoother="chebyshev", pre=3, post=3)
    mg = _mg(ctx, Ps, smoother="chebyshev")
    mg.update(U.SparseMatrix(ctx, A))
    z = U.Vector(ctx, n=A.nrows)
    mg.vcycle(U.Vector(ctx, b), z)
    assert rel(z.numpy(), omg.vcycle(b)) <= 1e-11


@pytest.mark.parametrize("precision", [U.F32, U.BF16])
def test_mixed_precision_fcg(ctx, oracle, precision):
    """Mixed form: FP32 V-cycle (Jacobi 0.8, 2+2) with FP32/BF16 level storage inside FP64
    flexible CG; relative residual 1e-8 checked in FP64, and the error against the FP64
    oracle solution reported."""
    A, Ps, b = P.lognormal_mg(48, 4, seed=2)
    nb = np.linalg.norm(b)
    Am = oracle.Matrix(A)
    x64, _ = oracle.cg_solve(Am, b, precond="mg",
                             mg=oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8),
                             atol=1e-12 * nb)
    mg = _mg(ctx, Ps, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
             precision=precision)
    s = cg(ctx, mg, atol=1e-8 * nb, flexible=1)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xg = x.numpy()
    assert np.linalg.norm(b - A.matvec(xg)) <= 1e-8 * nb * 1.0001
    assert rel(xg, x64) <= 1e-6


@pytest.mark.parametrize("shape", [(1, 1), (8, 8), (40, 25), (33, 63)])
def test_cholesky_solver_block_sizes(ctx, shape):
    """The blocked factorisation and inversion on sizes that are not multiples of the block (64)."""
    A = P.laplacian_2d(*shape)
    b = np.random.default_rng(1).standard_normal(A.nrows)
    x = U.Vector(ctx, n=A.nrows)
    U.CholeskySolver(ctx).solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xr = np.linalg.solve(A.to_scipy().toarray(), b)
    assert rel(x.numpy(), xr) <= 1e-12


def test_cholesky_solver_factored_inverse_above_4096(ctx):
    """Coarse sizes above 4096 keep the inverse factored (Y = L^-1 and Y^T in one buffer, two
    triangular GEMVs per solve): FP64 and FP32 vectors against a direct solve."""
    import scipy.sparse.linalg as spla
    A = P.laplacian_2d(71, 73)  # 5183 rows
    b = np.random.default_rng(2).standard_normal(A.nrows)
    s = U.CholeskySolver(ctx)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xr = spla.spsolve(A.to_scipy().tocsc(), b)
    assert rel(x.numpy(), xr) <= 1e-11
    b32 = b.astype(np.float32)
    x32 = U.Vector(ctx, n=A.nrows, dtype=U.F32)
    s.apply(U.Vector(ctx, b32, dtype=U.F32), x32)
    xr32 = spla.spsolve(A.to_scipy().tocsc(), b32.astype(np.float64))
    assert rel(x32.numpy().astype(np.float64), xr32) <= 1e-6


def test_cholesky_solver_and_not_spd(ctx):
    A = P.lognormal_diffusion_3d(9, 3)[0]
    b = np.random.default_rng(0).standard_normal(A.nrows)
    s = U.CholeskySolver(ctx)
    x = U.Vector(ctx, n=A.nrows)
    s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xr = np.linalg.solve(A.to_scipy().toarray(), b)
    assert rel(x.numpy(), xr) <= 1e-12
    Aneg = P.CSR(A.nrows, A.ncols, A.rowptr, A.colidx, -A.values)
    with pytest.raises(U.UgpuError) as e:
        U.CholeskySolver(ctx).update(U.SparseMatrix(ctx, Aneg))
    assert e.value.code == -4


@pytest.mark.parametrize("coarse_fp32", [0, 1])
def test_mixed_coarse_solve_precision(ctx, oracle, coarse_fp32):
    """The mixed V-cycle's coarse solve runs in FP64 (FP64 inverse and accumulation, FP32 vectors)
    by default; coarse_fp32 = 1 applies an FP32 copy of the inverse.  Both reach 1e-8 (FP64
    residual) and the FP64 oracle solution."""
    A, Ps, b = P.lognormal_mg(48, 4, seed=2)
    nb = np.linalg.norm(b)
    Am = oracle.Matrix(A)
    x64, _ = oracle.cg_solve(Am, b, precond="mg",
                             mg=oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8),
                             atol=1e-12 * nb)
    mg = _mg(ctx, Ps, smoother="jacobi", omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
             precision=U.BF16, coarse_fp32=coarse_fp32)
    s = cg(ctx, mg, atol=1e-8 * nb, flexible=1)
    x = U.Vector(ctx, n=A.nrows)
    assert s.solve(U.SparseMatrix(ctx, A), U.Vector(ctx, b), x)
    xg = x.numpy()
    assert np.linalg.norm(b - A.matvec(xg)) <= 1e-8 * nb
    assert rel(xg, x64) <= 1e-6


@pytest.mark.parametrize("smoother,precision,flexible",
                         [("jacobi", U.F64, 0), ("point_jacobi", U.F64, 0), ("jacobi", U.F32, 1),
                          ("jacobi", U.BF16, 1)])
def test_folded_outer_dots(ctx, oracle, smoother, precision, flexible):
    """fold_dots = 1: the V-cycle's last Jacobi sweep computes CG's (z, r) [and (z, Ap)] while it
    writes z.  Same iterations as the separate dot kernel (fold_dots = 0), solutions within
    round-off of each other, the FP64 form within 1e-9 of the oracle, and graph and eager runs
    bit-identical."""
    A, Ps, b = P.lognormal_mg(32, 3, seed=2)
    nb = np.linalg.norm(b)
    atol = (1e-10 if precision == U.F64 else 1e-8) * nb
    Am = U.SparseMatrix(ctx, A)
    out = {}
    for fold, graphs in ((0, 1), (1, 1), (1, 0)):
        mg = _mg(ctx, Ps, smoother=smoother, omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                 precision=precision)
        s = cg(ctx, mg, atol=atol, flexible=flexible, fold_dots=fold, use_graphs=graphs)
        x = U.Vector(ctx, n=A.nrows)
        assert s.solve(Am, U.Vector(ctx, b), x)
        out[(fold, graphs)] = (x.numpy(), s.solution_status()["iterates"])
    (x0, i0), (x1, i1), (x2, i2) = out[(0, 1)], out[(1, 1)], out[(1, 0)]
    assert abs(i1 - i0) <= 1
    assert i1 == i2 and np.array_equal(x1, x2)
    assert rel(x1, x0) <= (1e-9 if precision == U.F64 else 1e-6)
    assert np.linalg.norm(b - A.matvec(x1)) <= atol * 1.0001
    if precision == U.F64:
        Ao = oracle.Matrix(A)
        xo, so = oracle.cg_solve(Ao, b, precond="mg",
                                 mg=oracle.Multigrid(Ao, Ps, smoother=smoother, pre=2, post=2, omega=0.8),
                                 atol=atol)
        assert abs(i1 - so["iterates"]) <= 1
        assert rel(x1, xo) <= 1e-9


@pytest.mark.parametrize("smoother,precision,flexible",
                         [("jacobi", U.F64, 0), ("point_jacobi", U.F64, 0), ("jacobi", U.BF16, 1)])
def test_first_jacobi_iterate_from_the_producer(ctx, oracle, smoother, precision, flexible):
    """x1_from_producer = 1: the restriction (coarser levels) and CG's residual update (fine level)
    write the first Jacobi iterate w .* r beside r, and the pre-smoothing starts from the stored
    x1.  Against x1_from_producer = 0 (w_j r_j formed in every gather): the same iterations and
    x to rounding (the fused form lets the compiler contract the row's w_i r_i into an FMA);
    graph and eager runs bit-identical; the FP64 form within 1e-9 of the oracle, whose Jacobi
    stores x1 as well."""
    A, Ps, b = P.lognormal_mg(32, 3, seed=2)
    nb = np.linalg.norm(b)
    Am = U.SparseMatrix(ctx, A)
    out = []
    for prod, graphs in ((0, 1), (1, 1), (1, 0)):
        mg = _mg(ctx, Ps, smoother=smoother, omega=0.8, pre_smoothing_steps=2, post_smoothing_steps=2,
                 precision=precision, x1_from_producer=prod)
        s = cg(ctx, mg, atol=1e-10 * nb, flexible=flexible, use_graphs=graphs)
        x = U.Vector(ctx, n=A.nrows)
        assert s.solve(Am, U.Vector(ctx, b), x)
        out.append((x.numpy(), s.solution_status()["iterates"]))
    (x0, i0), (x1, i1), (x2, i2) = out
    assert i1 == i0 and i2 == i1
    assert np.array_equal(x2, x1)
    assert rel(x1, x0) <= (1e-12 if precision == U.F64 else 1e-6)
    if precision == U.F64:
        Ao = oracle.Matrix(A)
        xo, so = oracle.cg_solve(Ao, b, precond="mg",
                                 mg=oracle.Multigrid(Ao, Ps, smoother=smoother, pre=2, post=2, omega=0.8),
                                 atol=1e-10 * nb)
        assert abs(i1 - so["iterates"]) <= 1
        assert rel(x1, xo) <= 1e-9
