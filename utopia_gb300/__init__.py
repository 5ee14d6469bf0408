"""utopia_gb300 -- GB300 (sm_103a) backend for utopia's sparse-solver hot path.

Python front-end over the C ABI of ``libugpu.so`` (declared in ``include/ugpu.h``).
Class and method names follow the reference's C++ classes (``utopia::ConjugateGradient``,
``utopia::Multigrid``, ``utopia::InvDiagPreconditioner``, ``utopia::MPRGP``,
``utopia::ProjectedGaussSeidel``) so code written against them reads the same.
All numerical work runs in the library's CUDA kernels; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import BF16, F32, F64, FORMAT_CSR, FORMAT_SELL, UgpuError, check

__all__ = [
    "Context", "Vector", "SparseMatrix", "ConjugateGradient", "Multigrid", "InvDiagPreconditioner",
    "CholeskySolver", "MPRGP", "ProjectedGaussSeidel", "F64", "F32", "BF16", "UgpuError",
]

_NP = {F64: np.float64, F32: np.float32}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One device + one CUDA stream (the library's ``ugpu_ctx``)."""

    def __init__(self, device: int = 0):
        self.lib = _abi.load()
        h = C.c_void_p()
        check(self.lib.ugpu_create(int(device), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.ugpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        check(rc, self.h)

    def synchronize(self):
        self.check(self.lib.ugpu_synchronize(self.h))

    def launch_count(self) -> int:
        v = C.c_int64()
        self.check(self.lib.ugpu_launch_count(self.h, C.byref(v)))
        return v.value

    def fp64_rate(self, kind: str = "dfma") -> float:
        """Measured FP64 FLOP/s of this GPU: "dfma" (FMA chains) or "dmma" (FP64 mma.sync)."""
        v = C.c_double()
        self.check(self.lib.ugpu_fp64_rate(self.h, {"dfma": 0, "dmma": 1}[kind], C.byref(v)))
        return v.value

    @property
    def stream(self) -> int:
        v = C.c_void_p()
        self.check(self.lib.ugpu_stream(self.h, C.byref(v)))
        return v.value or 0

    # convenience constructors
    def vector(self, data=None, n=None, dtype=F64) -> "Vector":
        return Vector(self, data=data, n=n, dtype=dtype)

    def matrix(self, csr) -> "SparseMatrix":
        return SparseMatrix(self, csr)


class Vector:
    """Device vector (``ugpu_vec``); FP64 or FP32."""

    def __init__(self, ctx: Context, data=None, n=None, dtype=F64, _handle=None):
        self.ctx = ctx
        lib = ctx.lib
        if _handle is not None:
            self.h = _handle
        else:
            if data is not None:
                data = np.ascontiguousarray(data, dtype=_NP[dtype])
                n = data.size
            h = C.c_void_p()
            ctx.check(lib.ugpu_vec_create(ctx.h, int(n), int(dtype), C.byref(h)))
            self.h = h
            if data is not None:
                ctx.check(lib.ugpu_vec_upload(self.h, _ptr(data)))
        n_, dt = C.c_int64(), C.c_int()
        ctx.check(lib.ugpu_vec_size(self.h, C.byref(n_), C.byref(dt)))
        self.n, self.dtype = n_.value, dt.value

    @classmethod
    def wrap_device(cls, ctx, ptr: int, n: int, dtype=F64):
        h = C.c_void_p()
        ctx.check(ctx.lib.ugpu_vec_wrap_device(ctx.h, C.c_void_p(ptr), int(n), int(dtype), C.byref(h)))
        return cls(ctx, _handle=h)

    def __del__(self):
        try:
            self.ctx.lib.ugpu_vec_destroy(self.h)
        except Exception:
            pass

    def __len__(self):
        return self.n

    @property
    def device_ptr(self) -> int:
        v = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_vec_device_ptr(self.h, C.byref(v)))
        return v.value or 0

    def numpy(self):
        out = np.empty(self.n, dtype=_NP[self.dtype])
        self.ctx.check(self.ctx.lib.ugpu_vec_download(self.h, _ptr(out)))
        return out

    def write_petsc(self, path: str):
        self.ctx.check(self.ctx.lib.ugpu_petsc_write_vec(self.h, str(path).encode()))

    def write_raw(self, path: str):
        self.ctx.check(self.ctx.lib.ugpu_raw_vec_write(self.h, str(path).encode()))

    def upload_from(self, host_ptr: int):
        """Copy n elements from host memory at host_ptr (e.g. pinned) into the vector."""
        self.ctx.check(self.ctx.lib.ugpu_vec_upload(self.h, C.c_void_p(host_ptr)))

    def download_to(self, host_ptr: int):
        self.ctx.check(self.ctx.lib.ugpu_vec_download(self.h, C.c_void_p(host_ptr)))

    def upload(self, data):
        data = np.ascontiguousarray(data, dtype=_NP[self.dtype])
        assert data.size == self.n
        self.ctx.check(self.ctx.lib.ugpu_vec_upload(self.h, _ptr(data)))

    def set(self, value: float):
        self.ctx.check(self.ctx.lib.ugpu_vec_set(self.h, float(value)))

    def copy_to(self, other: "Vector"):
        self.ctx.check(self.ctx.lib.ugpu_vec_copy(self.h, other.h))

    def axpby(self, alpha, x: "Vector", beta):
        """self = alpha * x + beta * self"""
        self.ctx.check(self.ctx.lib.ugpu_axpby(float(alpha), x.h, float(beta), self.h))

    def dot(self, other: "Vector") -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.lib.ugpu_dot(self.h, other.h, C.byref(v)))
        return v.value

    def norm2(self) -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.lib.ugpu_norm2(self.h, C.byref(v)))
        return v.value


def dots(pairs):
    """utopia::dots -- several dots in one fused pass."""
    ctx = pairs[0][0].ctx
    k = len(pairs)
    a = (C.c_void_p * k)(*[p[0].h.value if isinstance(p[0].h, C.c_void_p) else p[0].h for p in pairs])
    b = (C.c_void_p * k)(*[p[1].h.value if isinstance(p[1].h, C.c_void_p) else p[1].h for p in pairs])
    out = (C.c_double * k)()
    ctx.check(ctx.lib.ugpu_dots(k, a, b, out))
    return list(out)


SET_ACTIVE, SET_FREE = 0, 1
RED_SUM, RED_MIN, RED_MAX, RED_ASUM, RED_AMAX = 0, 1, 2, 3, 4


def active_set(x: Vector, lb: Vector | None, ub: Vector | None, which=SET_ACTIVE):
    """Indices (ascending, int32) of the active (|l - x| < 1e-14 or |u - x| < 1e-14) or free
    (l < x < u) set of x, compacted on the device (ugpu_active_set_compact)."""
    import torch

    ctx = x.ctx
    buf = torch.empty(max(x.n, 1), dtype=torch.int32, device=torch.device("cuda", torch.cuda.current_device()))
    cnt = C.c_int64()
    ctx.check(ctx.lib.ugpu_active_set_compact(x.h, lb.h if lb is not None else None,
                                              ub.h if ub is not None else None, int(which),
                                              C.c_void_p(buf.data_ptr()), C.byref(cnt)))
    return buf[: cnt.value].cpu().numpy()


def reduce(v: Vector, op: int) -> float:
    """Reducible::reduce / Normed norms on the device (ugpu_vec_reduce): RED_SUM, RED_MIN, RED_MAX,
    RED_ASUM (norm1), RED_AMAX (norm_infty)."""
    out = C.c_double()
    v.ctx.check(v.ctx.lib.ugpu_vec_reduce(v.h, int(op), C.byref(out)))
    return out.value


class SparseMatrix:
    """Device CSR matrix (``ugpu_mat``) with its sliced-ELL SpMV layout."""

    def __init__(self, ctx: Context, csr=None, _handle=None):
        self.ctx = ctx
        lib = ctx.lib
        if _handle is not None:
            self.h = _handle
        else:
            rp = np.ascontiguousarray(csr.rowptr, dtype=np.int32)
            ci = np.ascontiguousarray(csr.colidx, dtype=np.int32)
            v = np.ascontiguousarray(csr.values, dtype=np.float64)
            h = C.c_void_p()
            ctx.check(lib.ugpu_csr_create(ctx.h, csr.nrows, csr.ncols, int(rp[-1]), _ptr(rp), _ptr(ci), _ptr(v),
                                          C.byref(h)))
            self.h = h
        n, m, nnz, dt = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
        ctx.check(lib.ugpu_mat_info(self.h, C.byref(n), C.byref(m), C.byref(nnz), C.byref(dt)))
        self.nrows, self.ncols, self.nnz, self.value_dtype = n.value, m.value, nnz.value, dt.value

    def __del__(self):
        try:
            self.ctx.lib.ugpu_mat_destroy(self.h)
        except Exception:
            pass

    @property
    def shape(self):
        return (self.nrows, self.ncols)

    def csr(self):
        """(rowptr, colidx, values as FP64) downloaded to the host."""
        rp = np.empty(self.nrows + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        v = np.empty(self.nnz, np.float64)
        self.ctx.check(self.ctx.lib.ugpu_csr_download(self.h, _ptr(rp), _ptr(ci), _ptr(v)))
        return rp, ci, v

    def cast(self, dtype) -> "SparseMatrix":
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_mat_cast(self.h, int(dtype), C.byref(h)))
        return SparseMatrix(self.ctx, _handle=h)

    def set_format(self, fmt):
        self.ctx.check(self.ctx.lib.ugpu_mat_set_format(self.h, int(fmt)))

    def sell_info(self):
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
        self.ctx.check(self.ctx.lib.ugpu_mat_sell_info(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"nslices": a.value, "nstored": b.value, "ndiag_slices": c.value, "rows_per_slice": d.value}

    def write_petsc(self, path: str):
        self.ctx.check(self.ctx.lib.ugpu_petsc_write_mat(self.h, str(path).encode()))

    def sell_interleaved(self) -> bool:
        """True when the sliced-ELL rows are lane-interleaved (the staged kernel's layout)."""
        v = C.c_int()
        self.ctx.check(self.ctx.lib.ugpu_mat_sell_layout(self.h, C.byref(v), None))
        return bool(v.value)

    def sell_anchored_slices(self) -> int:
        """Slices keyed by col - (first column of the row)."""
        v = C.c_int64()
        self.ctx.check(self.ctx.lib.ugpu_mat_sell_layout(self.h, None, C.byref(v)))
        return v.value

    def update_values(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.size == self.nnz
        self.ctx.check(self.ctx.lib.ugpu_mat_update_values(self.h, _ptr(v)))

    def diag(self, out: Vector):
        self.ctx.check(self.ctx.lib.ugpu_diag(self.h, out.h))

    def transpose(self) -> "SparseMatrix":
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_transpose(self.h, C.byref(h)))
        return SparseMatrix(self.ctx, _handle=h)

    def matmul(self, B: "SparseMatrix") -> "SparseMatrix":
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_spgemm(self.h, B.h, C.byref(h)))
        return SparseMatrix(self.ctx, _handle=h)

    def ptap(self, P: "SparseMatrix") -> "SparseMatrix":
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_ptap(self.h, P.h, C.byref(h)))
        return SparseMatrix(self.ctx, _handle=h)

    def ptap_reuse(self, P: "SparseMatrix", out: "SparseMatrix | None" = None) -> "SparseMatrix":
        """MatPtAP with MatReuse: without `out` a new product that keeps its structure
        (MAT_INITIAL_MATRIX); with `out` (such a product) its values recomputed in place for the
        current values of self and P (MAT_REUSE_MATRIX)."""
        if out is None:
            h = C.c_void_p()
            self.ctx.check(self.ctx.lib.ugpu_ptap_reuse(self.h, P.h, 0, C.byref(h)))
            return SparseMatrix(self.ctx, _handle=h)
        h = C.c_void_p(out.h.value if isinstance(out.h, C.c_void_p) else out.h)
        self.ctx.check(self.ctx.lib.ugpu_ptap_reuse(self.h, P.h, 1, C.byref(h)))
        return out

    # Operator::apply
    def apply(self, x: Vector, y: Vector):
        self.ctx.check(self.ctx.lib.ugpu_spmv(self.h, x.h, y.h))

    def apply_dot(self, x: Vector, y: Vector, out: Vector | None = None) -> float | None:
        """y = A x and (x, y) from one kernel.  With out (an FP64 vector), the dot is left in
        out[0] on the device and nothing is returned; without, it is returned as a float."""
        if out is not None:
            self.ctx.check(self.ctx.lib.ugpu_spmv_dot(self.h, x.h, y.h, out.h))
            return None
        d = Vector(self.ctx, n=1)
        self.ctx.check(self.ctx.lib.ugpu_spmv_dot(self.h, x.h, y.h, d.h))
        return float(d.numpy()[0])

    def apply_add(self, x: Vector, v: Vector, y: Vector):
        self.ctx.check(self.ctx.lib.ugpu_spmv_add(self.h, x.h, v.h, y.h))

    def residual(self, b: Vector, x: Vector, r: Vector):
        self.ctx.check(self.ctx.lib.ugpu_residual(self.h, b.h, x.h, r.h))

    def jacobi_sweep(self, b: Vector, x: Vector, omega: float, x_out: Vector):
        self.ctx.check(self.ctx.lib.ugpu_jacobi_sweep(self.h, b.h, x.h, float(omega), x_out.h))


def read_petsc_matrix(ctx: "Context", path: str) -> "SparseMatrix":
    """A PETSc binary matrix file (FP64 CSR on the device)."""
    h = C.c_void_p()
    ctx.check(ctx.lib.ugpu_petsc_read_mat(ctx.h, str(path).encode(), C.byref(h)))
    return SparseMatrix(ctx, _handle=h)


def read_petsc_vector(ctx: "Context", path: str) -> "Vector":
    h = C.c_void_p()
    ctx.check(ctx.lib.ugpu_petsc_read_vec(ctx.h, str(path).encode(), C.byref(h)))
    return Vector(ctx, _handle=h)


def read_raw_crs(ctx: "Context", directory: str, index_bytes=4, value_bytes=8, ncols=0) -> "SparseMatrix":
    """rowptr.raw, colidx.raw and values.raw of one directory."""
    h = C.c_void_p()
    ctx.check(ctx.lib.ugpu_raw_crs_read(ctx.h, str(directory).encode(), int(index_bytes), int(value_bytes),
                                        int(ncols), C.byref(h)))
    return SparseMatrix(ctx, _handle=h)


def read_raw_vector(ctx: "Context", path: str, value_bytes=8) -> "Vector":
    h = C.c_void_p()
    ctx.check(ctx.lib.ugpu_raw_vec_read(ctx.h, str(path).encode(), int(value_bytes), C.byref(h)))
    return Vector(ctx, _handle=h)


class _Solver:
    KIND = 0

    def __init__(self, ctx: Context, **params):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(ctx.lib.ugpu_solver_create(ctx.h, self.KIND, C.byref(h)))
        self.h = h
        self._keep = []
        for k, v in params.items():
            self.set(k, v)

    def __del__(self):
        try:
            self.ctx.lib.ugpu_solver_destroy(self.h)
        except Exception:
            pass

    def set(self, key, value):
        self.ctx.check(self.ctx.lib.ugpu_solver_set(self.h, key.encode(), float(value)))
        return self

    def get(self, key) -> float:
        v = C.c_double()
        self.ctx.check(self.ctx.lib.ugpu_solver_get(self.h, key.encode(), C.byref(v)))
        return v.value

    # IterativeSolver accessors
    def atol(self, v=None):
        return self.get("atol") if v is None else self.set("atol", v)

    def rtol(self, v=None):
        return self.get("rtol") if v is None else self.set("rtol", v)

    def stol(self, v=None):
        return self.get("stol") if v is None else self.set("stol", v)

    def max_it(self, v=None):
        return int(self.get("max_it")) if v is None else self.set("max_it", v)

    def update(self, A: SparseMatrix):
        self._keep.append(A)
        self._keep = self._keep[-1:]
        self.ctx.check(self.ctx.lib.ugpu_solver_update(self.h, A.h))

    def apply(self, rhs: Vector, x: Vector) -> bool:
        self.ctx.check(self.ctx.lib.ugpu_solver_apply(self.h, rhs.h, x.h))
        return bool(self.solution_status()["converged"])

    def solve(self, A: SparseMatrix, b: Vector, x: Vector) -> bool:
        self.update(A)
        return self.apply(b, x)

    def solution_status(self) -> dict:
        st = _abi.SolutionStatus()
        self.ctx.check(self.ctx.lib.ugpu_solver_status(self.h, C.byref(st)))
        return st.as_dict()


class InvDiagPreconditioner(_Solver):
    KIND = _abi.SOLVER_INVDIAG


class CholeskySolver(_Solver):
    KIND = _abi.SOLVER_CHOLESKY


class ConjugateGradient(_Solver):
    KIND = _abi.SOLVER_CG

    def set_preconditioner(self, prec):
        self._prec = prec
        self.ctx.check(self.ctx.lib.ugpu_solver_set_preconditioner(self.h, prec.h if prec is not None else None))


SMOOTHERS = {"jacobi": 0, "chebyshev": 1, "point_jacobi": 2}


class Multigrid(_Solver):
    KIND = _abi.SOLVER_MULTIGRID

    def __init__(self, ctx, smoother="chebyshev", precision=F64, **params):
        super().__init__(ctx, smoother=SMOOTHERS[smoother] if isinstance(smoother, str) else smoother,
                         precision=precision, **params)

    def set_transfer_operators(self, interpolations):
        mats = [p if isinstance(p, SparseMatrix) else SparseMatrix(self.ctx, p) for p in interpolations]
        arr = (C.c_void_p * len(mats))(*[m.h.value for m in mats])
        self.ctx.check(self.ctx.lib.ugpu_mg_set_transfer_operators(self.h, len(mats), arr))

    def pre_smoothing_steps(self, v):
        return self.set("pre_smoothing_steps", v)

    def post_smoothing_steps(self, v):
        return self.set("post_smoothing_steps", v)

    def n_levels(self) -> int:
        v = C.c_int()
        self.ctx.check(self.ctx.lib.ugpu_mg_n_levels(self.h, C.byref(v)))
        return v.value

    def level_matrix(self, l) -> SparseMatrix:
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.ugpu_mg_level_matrix(self.h, int(l), C.byref(h)))
        return SparseMatrix(self.ctx, _handle=h)

    def eigs(self, l):
        a, b = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.ugpu_mg_eigs(self.h, int(l), C.byref(a), C.byref(b)))
        return a.value, b.value

    def vcycle(self, r: Vector, z: Vector):
        self.ctx.check(self.ctx.lib.ugpu_mg_vcycle(self.h, r.h, z.h))


class AlgebraicMultigrid(Multigrid):
    """utopia::AlgebraicMultigrid with utopia::Agglomerate: the hierarchy is built from the
    operator by greedy aggregation (keys n_levels, bmax, weight, use_additive_correction;
    n_levels=0 coarsens until at most max_coarse_rows rows), then runs as the multigrid."""

    KIND = _abi.SOLVER_AMG

    def set_transfer_operators(self, interpolations):
        raise TypeError("the algebraic multigrid builds its own transfer operators")

    def parent(self, level: int):
        """Aggregate of every row of level `level` (0 = the fine operator); -2 = excluded row."""
        n, nc = C.c_int64(), C.c_int64()
        self.ctx.check(self.ctx.lib.ugpu_amg_parent(self.h, int(level), None, C.byref(n), C.byref(nc)))
        out = np.empty(n.value, np.int32)
        self.ctx.check(self.ctx.lib.ugpu_amg_parent(self.h, int(level), _ptr(out), None, None))
        return out, nc.value


class BiCGStab(_Solver):
    """utopia::BiCGStab; preconditioned when a (FP64) preconditioner is set."""

    KIND = _abi.SOLVER_BICGSTAB

    def set_preconditioner(self, prec):
        self._prec = prec
        self.ctx.check(self.ctx.lib.ugpu_solver_set_preconditioner(self.h, prec.h))


class _QPSolver(_Solver):
    def set_box_constraints(self, lb: Vector | None, ub: Vector | None):
        self._box = (lb, ub)
        self.ctx.check(self.ctx.lib.ugpu_qp_set_box_constraints(self.h, lb.h if lb is not None else None,
                                                                ub.h if ub is not None else None))


class SemismoothNewton(_QPSolver):
    """utopia::SemismoothNewton (primal-dual active set); set_linear_solver replaces the default
    inner BiCGStab + Jacobi."""

    KIND = _abi.SOLVER_SSNEWTON

    def set_linear_solver(self, solver):
        self._linear = solver
        self.ctx.check(self.ctx.lib.ugpu_solver_set_preconditioner(self.h, solver.h))


class ShiftedPenaltyQPSolver(_QPSolver):
    """utopia::ShiftedPenaltyQPSolver with utopia::ShiftedPenalty: the upper bound is enforced by a
    shifted quadratic penalty, one linear solve per iteration (as in the reference, a lower bound
    alone is inert: the missing upper bound is filled with the largest double).  Keys
    penalty_parameter, penalty_parameter_max, penalty_parameter_factor, zero_shift_on_reset,
    linear_rtol, linear_max_it).  set_linear_solver replaces the default inner CG + Jacobi;
    set_transform(T, O), set_selection and set_scaling_matrix add the optional terms."""

    KIND = _abi.SOLVER_SHIFTED_PENALTY

    def set_linear_solver(self, solver):
        self._linear = solver
        self.ctx.check(self.ctx.lib.ugpu_solver_set_preconditioner(self.h, solver.h))

    def set_transform(self, T: SparseMatrix | None, O: SparseMatrix | None):
        self._trafo = (T, O)
        self.ctx.check(self.ctx.lib.ugpu_penalty_set_transform(self.h, T.h if T is not None else None,
                                                               O.h if O is not None else None))

    def set_selection(self, selection: Vector | None):
        self._selection = selection
        self.ctx.check(self.ctx.lib.ugpu_penalty_set_selection(self.h, selection.h if selection is not None else None))

    def set_scaling_matrix(self, S: SparseMatrix | None):
        self._scaling = S
        self.ctx.check(self.ctx.lib.ugpu_penalty_set_scaling_matrix(self.h, S.h if S is not None else None))


class MPRGP(_QPSolver):
    KIND = _abi.SOLVER_MPRGP


class MonotoneMultigrid(_QPSolver):
    """utopia::MonotoneMultigrid: projected Gauss-Seidel on the fine level, the fine transfer
    truncated on the active set, a linear multigrid (smoother "jacobi", "chebyshev" or
    "point_jacobi") on the truncated Galerkin operator.  Interpolations are given coarse -> fine;
    the last one is the fine-level transfer."""

    KIND = _abi.SOLVER_MONOTONE_MG

    def __init__(self, ctx, smoother="chebyshev", **params):
        super().__init__(ctx, smoother=SMOOTHERS[smoother] if isinstance(smoother, str) else smoother, **params)

    set_transfer_operators = Multigrid.set_transfer_operators
    pre_smoothing_steps = Multigrid.pre_smoothing_steps
    post_smoothing_steps = Multigrid.post_smoothing_steps
    n_levels = Multigrid.n_levels
    level_matrix = Multigrid.level_matrix

    def active_set(self):
        """ActiveSet::indicator after the last update/apply (0/1 per fine dof)."""
        na = C.c_int64()
        self.ctx.check(self.ctx.lib.ugpu_mmg_active_set(self.h, None, C.byref(na)))
        out = np.empty(self._keep[-1].nrows, np.int32)
        self.ctx.check(self.ctx.lib.ugpu_mmg_active_set(self.h, _ptr(out), None))
        return out


class ProjectedGaussSeidel(_QPSolver):
    KIND = _abi.SOLVER_PGS

    def colouring(self):
        nc = C.c_int()
        self.ctx.check(self.ctx.lib.ugpu_pgs_colouring(self.h, None, C.byref(nc)))
        n = self._keep[-1].nrows
        out = np.empty(n, np.int32)
        self.ctx.check(self.ctx.lib.ugpu_pgs_colouring(self.h, _ptr(out), C.byref(nc)))
        return out, nc.value
