"""Differentiable solve: assembly and gradient kernels against the oracle, gradcheck and
central finite differences in FP64 at 16^3, and the mixed-precision gradient at 128^3
against the CPU FP64 gradient."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def oracle_solve(oracle, A, Ps, b, rtol=1e-12):
    Am = oracle.Matrix(A)
    mg = oracle.Multigrid(Am, Ps, smoother="jacobi", pre=2, post=2, omega=0.8)
    x, st = oracle.cg_solve(Am, b, precond="mg", mg=mg, atol=rtol * np.linalg.norm(b), max_it=500)
    assert st["converged"]
    return x


def test_graph_assemble_and_gradient_kernels(ctx, oracle):
    from utopia_gb300.autograd import Graph, pattern_grad

    G = P.EdgeGraph(10)
    rng = np.random.default_rng(0)
    theta = rng.normal(0, 0.5, G.E)
    A_ref = G.assemble(theta)
    graph = Graph(ctx, G.n, G.src, G.dst, G.edge_of_pos(), G.nbnd)
    A = U.SparseMatrix(ctx, G.assemble(np.zeros(G.E)))
    for dt, npdt in ((U.F64, np.float64), (U.F32, np.float32)):
        th = U.Vector(ctx, theta.astype(npdt), dtype=dt)
        graph.assemble(th, A)
        _, _, v = A.csr()
        ref = G.assemble(theta.astype(npdt).astype(np.float64)).values
        np.testing.assert_allclose(v, ref, rtol=1e-14, atol=1e-14)
        lam, x = rng.standard_normal(G.n), rng.standard_normal(G.n)
        grad = U.Vector(ctx, n=G.E, dtype=dt)
        graph.edge_grad(th, U.Vector(ctx, lam), U.Vector(ctx, x), grad)
        if dt == U.F32:
            gref = oracle.edge_grad(G.src, G.dst, theta.astype(np.float32), lam, x)
            tol = 1e-6
        else:
            gref = -np.exp(theta) * (lam[G.src] - lam[G.dst]) * (x[G.src] - x[G.dst])
            tol = 1e-13
        np.testing.assert_allclose(grad.numpy(), gref, rtol=tol, atol=tol * np.abs(gref).max())
    gv = U.Vector(ctx, n=A.nnz)
    pattern_grad(A, U.Vector(ctx, lam), U.Vector(ctx, x), gv)
    np.testing.assert_allclose(gv.numpy(), oracle.pattern_grad(oracle.Matrix(A_ref), lam, x), rtol=1e-15)


def make_solver(ctx, N, precision=U.F64, rtol=1e-13):
    from utopia_gb300.autograd import DifferentiableGraphSolver

    G, theta, b, theta_t = P.graph_adjoint(N)
    levels = 3 if N <= 32 else 4
    Ps = P.hierarchy_3d(N, levels)
    return G, theta, b, theta_t, Ps, DifferentiableGraphSolver(ctx, G, Ps, precision=precision, rtol=rtol)


def test_gradcheck_fp64_16(ctx, oracle):
    """torch.autograd.gradcheck through GraphSolve on a 16^3 instance in FP64: the loss
    L = ||x - x_target||^2 restricted to a random 6-dimensional subspace of theta and a
    4-dimensional subspace of b (central differences)."""
    from utopia_gb300.autograd import GraphSolve

    G, theta, b, theta_t, Ps, solver = make_solver(ctx, 16)
    x_t = torch.from_numpy(oracle_solve(oracle, G.assemble(theta_t), Ps, b))
    rng = np.random.default_rng(1)
    V = torch.from_numpy(rng.standard_normal((G.E, 6)) * 0.05)
    W = torch.from_numpy(rng.standard_normal((G.n, 4)) * 0.01)
    th0 = torch.from_numpy(theta.astype(np.float64))
    b0 = torch.from_numpy(b)

    def loss(s, t):
        x = GraphSolve.apply(th0 + V @ s, b0 + W @ t, solver)
        return ((x - x_t) ** 2).sum()

    s = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    t = torch.zeros(4, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(loss, (s, t), eps=1e-6, atol=1e-9, rtol=1e-6)


def test_adjoint_matches_central_differences(ctx, oracle):
    """Directional derivatives dL/dtheta . v from the adjoint against central finite
    differences of L (FP64 solves at 1e-13), relative agreement 1e-6."""
    from utopia_gb300.autograd import GraphSolve

    G, theta, b, theta_t, Ps, solver = make_solver(ctx, 16)
    x_t = torch.from_numpy(oracle_solve(oracle, G.assemble(theta_t), Ps, b))
    th = torch.from_numpy(theta.astype(np.float64)).requires_grad_(True)
    bt = torch.from_numpy(b).requires_grad_(True)
    L = ((GraphSolve.apply(th, bt, solver) - x_t) ** 2).sum()
    L.backward()
    rng = np.random.default_rng(2)

    def Lval(thv, bv):
        with torch.no_grad():
            return float(((GraphSolve.apply(thv, bv, solver) - x_t) ** 2).sum())

    for k in range(4):
        v = torch.from_numpy(rng.standard_normal(G.E))
        h = 1e-4
        fd = (Lval(th.detach() + h * v, bt.detach()) - Lval(th.detach() - h * v, bt.detach())) / (2 * h)
        ad = float(th.grad @ v)
        assert abs(ad - fd) <= 1e-6 * abs(fd), (k, ad, fd)
    w = torch.from_numpy(rng.standard_normal(G.n) * 0.01)
    h = 1e-3
    fd = (Lval(th.detach(), bt.detach() + h * w) - Lval(th.detach(), bt.detach() - h * w)) / (2 * h)
    assert abs(float(bt.grad @ w) - fd) <= 1e-6 * abs(fd)


def test_mixed_gradient_128_vs_cpu_fp64(ctx, oracle):
    """Forward with the mixed MG-PCG (BF16/FP32 V-cycle, FP64 flexible CG at 1e-8) at 128^3
    (6,242,304 edges, FP32 theta); dL/dtheta and dL/db against the CPU FP64 gradient."""
    from utopia_gb300.autograd import GraphSolve

    G, theta, b, theta_t, Ps, solver = make_solver(ctx, 128, precision=U.BF16, rtol=1e-8)
    x_t = oracle_solve(oracle, G.assemble(theta_t), Ps, b, rtol=1e-11)
    # CPU FP64 reference gradient
    A = G.assemble(theta)
    x_ref = oracle_solve(oracle, A, Ps, b, rtol=1e-11)
    lam_ref = oracle_solve(oracle, A, Ps, 2 * (x_ref - x_t), rtol=1e-11)
    g_ref = oracle.edge_grad(G.src, G.dst, theta, lam_ref, x_ref)
    dev = torch.device("cuda")
    th = torch.from_numpy(theta).to(dev).requires_grad_(True)
    bt = torch.from_numpy(b).to(dev).requires_grad_(True)
    x = GraphSolve.apply(th, bt, solver)
    L = ((x - torch.from_numpy(x_t).to(dev)) ** 2).sum()
    L.backward()
    assert th.grad.dtype == torch.float32
    g = th.grad.double().cpu().numpy()
    assert np.linalg.norm(g - g_ref) <= 1e-5 * np.linalg.norm(g_ref)
    lam = bt.grad.cpu().numpy()
    assert np.linalg.norm(lam - lam_ref) <= 1e-5 * np.linalg.norm(lam_ref)
    assert np.linalg.norm(x.detach().cpu().numpy() - x_ref) <= 1e-6 * np.linalg.norm(x_ref)
