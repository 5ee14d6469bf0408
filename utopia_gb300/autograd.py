"""Differentiable sparse solve x = A(theta)^{-1} b over the C ABI.

A(theta) = sum_e exp(theta_e) (e_i - e_j)(e_i - e_j)^T + diag(boundary) on a graph with
per-edge log-conductances.  The forward pass assembles A(theta) on the device, builds the
multigrid hierarchy and runs multigrid-preconditioned CG (plain FP64, or the mixed form:
BF16/FP32 V-cycle inside FP64 flexible CG).  The backward pass keeps only x: it solves
A^T lambda = dL/dx with the same solver and hierarchy (A is symmetric), and returns
dL/db = lambda and dL/dtheta_e = -exp(theta_e)(lambda_i - lambda_j)(x_i - x_j) from one
edge kernel.  There is no reference counterpart to this path.

``GraphSolve`` is a thin ``torch.autograd.Function`` over it; theta and b may be CPU or
CUDA tensors (CUDA tensors are read and written in place, without copies).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import BF16, F32, F64, ConjugateGradient, Multigrid, SparseMatrix, Vector, _abi


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Graph:
    """Device copy of the edge data of a problems.EdgeGraph-like description."""

    def __init__(self, ctx, n, src, dst, edge_of_pos, boundary):
        self.ctx = ctx
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        eop = np.ascontiguousarray(edge_of_pos, np.int32)
        bnd = np.ascontiguousarray(boundary, np.float64)
        self.n, self.E, self.nnz = int(n), int(src.size), int(eop.size)
        h = C.c_void_p()
        ctx.check(ctx.lib.ugpu_graph_create(ctx.h, self.n, self.E, _ptr(src), _ptr(dst), self.nnz, _ptr(eop),
                                            _ptr(bnd), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            self.ctx.lib.ugpu_graph_destroy(self.h)
        except Exception:
            pass

    def assemble(self, theta: Vector, A: SparseMatrix):
        self.ctx.check(self.ctx.lib.ugpu_graph_assemble(self.h, theta.h, A.h))

    def edge_grad(self, theta: Vector, lam: Vector, x: Vector, grad: Vector):
        self.ctx.check(self.ctx.lib.ugpu_graph_edge_grad(self.h, theta.h, lam.h, x.h, grad.h))


def pattern_grad(A: SparseMatrix, lam: Vector, x: Vector, out: Vector):
    """out[k] = -lambda_i x_j for every CSR entry k = (i, j) of A."""
    A.ctx.check(A.ctx.lib.ugpu_pattern_grad(A.h, lam.h, x.h, out.h))


class DifferentiableGraphSolver:
    """Forward solve, adjoint solve and edge gradient on one device context.

    precision: F64 (plain FP64 MG-PCG) or F32 / BF16 (mixed form, flexible CG outer loop).
    rtol: stop when ||r|| <= rtol ||rhs|| (FP64), for the forward and the adjoint solve.
    """

    def __init__(self, ctx, edge_graph, interpolations, precision=F64, rtol=1e-10, smoother="jacobi", omega=0.8,
                 pre=2, post=2, max_it=500):
        G = edge_graph
        self.ctx = ctx
        self.n, self.E = G.n, G.E
        self.graph = Graph(ctx, G.n, G.src, G.dst, G.edge_of_pos(), G.nbnd)
        self.A = SparseMatrix(ctx, G.assemble(np.zeros(G.E)))  # pattern; values set per forward
        self.mg = Multigrid(ctx, smoother=smoother, omega=omega, pre_smoothing_steps=pre,
                            post_smoothing_steps=post, precision=precision)
        self.mg.set_transfer_operators(interpolations)
        self.cg = ConjugateGradient(ctx, flexible=0 if precision == F64 else 1, max_it=max_it)
        self.cg.set_preconditioner(self.mg)
        self.rtol = rtol
        self.status = {}

    def _solve(self, rhs: Vector, x: Vector):
        nrm = rhs.norm2()
        x.set(0.0)
        if nrm == 0.0:  # A^{-1} 0 = 0 (CG itself would stop on 0/0, as the reference does)
            return {"iterates": 0, "converged": 1, "gradient_norm": 0.0}
        self.cg.atol(self.rtol * nrm)
        self.cg.apply(rhs, x)
        st = self.cg.solution_status()
        if not st["converged"]:
            raise RuntimeError(f"solve did not converge: {st}")
        return st

    def forward(self, theta: Vector, b: Vector, x: Vector):
        """x = A(theta)^{-1} b; builds the hierarchy for A(theta)."""
        self.graph.assemble(theta, self.A)
        self.cg.update(self.A)
        self.status["forward"] = self._solve(b, x)

    def adjoint(self, g: Vector, lam: Vector):
        """lambda = A^{-T} g with the forward pass's operator and hierarchy."""
        self.status["adjoint"] = self._solve(g, lam)

    def edge_grad(self, theta: Vector, lam: Vector, x: Vector, grad: Vector):
        self.graph.edge_grad(theta, lam, x, grad)


def _as_vector(ctx, t, dtype):
    """A library vector viewing a contiguous CUDA tensor, or a device copy of a CPU tensor."""
    import torch

    want = torch.float64 if dtype == F64 else torch.float32
    if t.is_cuda:
        t = t.detach().to(want).contiguous()
        return Vector.wrap_device(ctx, t.data_ptr(), t.numel(), dtype), t
    return Vector(ctx, t.detach().to(want).numpy(), dtype=dtype), None


def _out_tensor(vec, like, dtype):
    import torch

    want = torch.float64 if dtype == F64 else torch.float32
    if like.is_cuda:
        out = torch.empty(vec.n, dtype=want, device=like.device)
        tmp = Vector.wrap_device(vec.ctx, out.data_ptr(), vec.n, dtype)
        vec.copy_to(tmp)
        vec.ctx.synchronize()
        return out
    return torch.from_numpy(vec.numpy()).to(want)


try:
    import torch

    class GraphSolve(torch.autograd.Function):
        """x = GraphSolve.apply(theta, b, solver) with an adjoint backward."""

        @staticmethod
        def forward(ctx, theta, b, solver: DifferentiableGraphSolver):
            if theta.is_cuda or b.is_cuda:
                torch.cuda.synchronize()
            tdt = F64 if theta.dtype == torch.float64 else F32
            th_v, th_keep = _as_vector(solver.ctx, theta, tdt)
            b_v, b_keep = _as_vector(solver.ctx, b, F64)
            x_v = Vector(solver.ctx, n=solver.n)
            solver.forward(th_v, b_v, x_v)
            ctx.solver = solver
            ctx.tdt = tdt
            ctx.x_v = x_v  # the only state the backward pass keeps besides theta
            ctx.save_for_backward(theta)
            return _out_tensor(x_v, b, F64)

        @staticmethod
        def backward(ctx, grad_x):
            (theta,) = ctx.saved_tensors
            solver = ctx.solver
            if grad_x.is_cuda:
                torch.cuda.synchronize()
            g_v, g_keep = _as_vector(solver.ctx, grad_x, F64)
            lam = Vector(solver.ctx, n=solver.n)
            solver.adjoint(g_v, lam)
            th_v, th_keep = _as_vector(solver.ctx, theta, ctx.tdt)
            grad = Vector(solver.ctx, n=solver.E, dtype=ctx.tdt)
            solver.edge_grad(th_v, lam, ctx.x_v, grad)
            grad_theta = _out_tensor(grad, theta, ctx.tdt).to(theta.dtype)
            grad_b = _out_tensor(lam, grad_x, F64)
            return grad_theta, grad_b, None

except ImportError:  # pragma: no cover
    GraphSolve = None
