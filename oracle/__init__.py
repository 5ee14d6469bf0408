"""ctypes front-end of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, always as the checker or the timed CPU
reference, never as part of the GPU product path.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.cpp into liboracle.so (g++, OpenMP, portable flags)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", _SO + ".tmp", src]
        subprocess.check_call(cmd)
        os.replace(_SO + ".tmp", _SO)
    return _SO


class Status(C.Structure):
    _fields_ = [
        ("iterates", C.c_int64),
        ("gradient_norm", C.c_double),
        ("relative_gradient_norm", C.c_double),
        ("step_norm", C.c_double),
        ("reason", C.c_int32),
        ("converged", C.c_int32),
        ("spmv_count", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_vp = C.c_void_p
_d = C.c_double
_i64 = C.c_int64
_i32 = C.c_int32


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            sig = {
                "or_set_threads": (None, [C.c_int]),
                "or_max_threads": (C.c_int, []),
                "or_glibc_rand": (None, [C.c_uint32, _i64, _vp]),
                "or_csr_create": (_vp, [_i64, _i64, _vp, _vp, _vp]),
                "or_csr_free": (None, [_vp]),
                "or_csr_info": (None, [_vp, _vp, _vp, _vp]),
                "or_csr_get": (None, [_vp, _vp, _vp, _vp]),
                "or_spmv": (None, [_vp, _vp, _vp]),
                "or_residual": (None, [_vp, _vp, _vp, _vp]),
                "or_dot": (_d, [_i64, _vp, _vp]),
                "or_transpose": (_vp, [_vp]),
                "or_spgemm": (_vp, [_vp, _vp]),
                "or_ptap": (_vp, [_vp, _vp]),
                "or_cg_solve": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, _d, _d, _d, _i64, C.c_int, _vp]),
                "or_mg_create": (_vp, [_vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _d, C.c_int, C.c_int]),
                "or_mg_free": (None, [_vp]),
                "or_mg_levels": (C.c_int, [_vp]),
                "or_mg_level_matrix": (_vp, [_vp, C.c_int]),
                "or_mg_eigs": (None, [_vp, C.c_int, _vp, _vp]),
                "or_mg_mask": (None, [_vp, C.c_int, _vp]),
                "or_mg_vcycle": (None, [_vp, _vp, _vp]),
                "or_mg_solve": (C.c_int, [_vp, _vp, _vp, _d, _d, _i64, _vp]),
                "or_mprgp_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _d, _d, _i64, _d, _i64, _vp, _vp]),
                "or_pgs_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _d, _i64, C.c_int, C.c_int, _vp, C.c_int, _vp]),
                "or_colouring": (C.c_int, [_vp, _vp]),
                "or_projected_gradient_norm": (_d, [_vp, _vp, _vp, _vp, _vp]),
                "or_edge_grad": (None, [_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
                "or_pattern_grad": (None, [_vp, _vp, _vp, _vp]),
                "or_agglomerate": (_vp, [_vp, _i64, _d, C.c_int, _vp]),
                "or_bicgstab_solve": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, _d, _i64, _vp]),
                "or_ssn_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _d, _i64, _d, _vp]),
                "or_penalty_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _vp,
                                               C.c_int, _d, _i64, _d, _i64, _vp]),
                "or_mmg_solve": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_int, C.c_int, _d, _d, C.c_int, _d, _d, _d, _i64, _vp,
                                           _vp, _vp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(t: int):
    lib().or_set_threads(int(t))


def max_threads() -> int:
    return lib().or_max_threads()


def glibc_rand(count: int, seed: int = 1):
    out = np.empty(count, dtype=np.int32)
    lib().or_glibc_rand(seed, count, _p(out))
    return out


class Matrix:
    """Oracle-owned FP64 CSR matrix."""

    def __init__(self, csr=None, _handle=None):
        L = lib()
        if _handle is not None:
            self.h = _handle
        else:
            rp = np.ascontiguousarray(csr.rowptr, dtype=np.int32)
            ci = np.ascontiguousarray(csr.colidx, dtype=np.int32)
            v = _f64(csr.values)
            self.h = L.or_csr_create(csr.nrows, csr.ncols, _p(rp), _p(ci), _p(v))
        n, m, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        L.or_csr_info(self.h, C.byref(n), C.byref(m), C.byref(nnz))
        self.nrows, self.ncols, self.nnz = n.value, m.value, nnz.value

    def __del__(self):
        try:
            lib().or_csr_free(self.h)
        except Exception:
            pass

    def arrays(self):
        rp = np.empty(self.nrows + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        v = np.empty(self.nnz, np.float64)
        lib().or_csr_get(self.h, _p(rp), _p(ci), _p(v))
        return rp, ci, v

    def matvec(self, x):
        x = _f64(x)
        y = np.empty(self.nrows)
        lib().or_spmv(self.h, _p(x), _p(y))
        return y

    def transpose(self):
        return Matrix(_handle=lib().or_transpose(self.h))

    def matmul(self, other):
        return Matrix(_handle=lib().or_spgemm(self.h, other.h))

    def ptap(self, P):
        return Matrix(_handle=lib().or_ptap(self.h, P.h))


def dot(a, b) -> float:
    a = _f64(a)
    b = _f64(b)
    return lib().or_dot(a.size, _p(a), _p(b))


def cg_solve(A: Matrix, b, x0=None, precond="invdiag", mg=None, atol=1e-9, rtol=1e-9, stol=1e-11,
             max_it=1000, flexible=False):
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    kind = {"none": 0, "invdiag": 1, "mg": 2}[precond]
    lib().or_cg_solve(A.h, _p(b), _p(x), kind, mg.h if mg is not None else None, atol, rtol, stol,
                      max_it, int(flexible), C.byref(st))
    return x, st.as_dict()


SMOOTHERS = {"jacobi": 0, "chebyshev": 1, "point_jacobi": 2}
PRECISIONS = {"fp64": 0, "fp32": 1, "bf16": 2}


class Multigrid:
    def __init__(self, A: Matrix, P_coarse_to_fine, precision="fp64", smoother="chebyshev", pre=3, post=3,
                 omega=1.0, fix_semidefinite=False, masks=True):
        self._P = [p if isinstance(p, Matrix) else Matrix(p) for p in P_coarse_to_fine]
        arr = (C.c_void_p * len(self._P))(*[p.h for p in self._P])
        self.h = lib().or_mg_create(A.h, len(self._P), C.cast(arr, C.c_void_p), PRECISIONS[precision],
                                    SMOOTHERS[smoother], pre, post, omega, int(fix_semidefinite), int(masks))
        if not self.h:
            raise RuntimeError("oracle multigrid set-up failed (coarse operator not SPD?)")
        self.n_levels = lib().or_mg_levels(self.h)
        self.sizes = [self.level_matrix(l).nrows for l in range(self.n_levels)]

    def __del__(self):
        try:
            lib().or_mg_free(self.h)
        except Exception:
            pass

    def level_matrix(self, l) -> Matrix:
        return Matrix(_handle=lib().or_mg_level_matrix(self.h, l))

    def eigs(self, l):
        a, b = C.c_double(), C.c_double()
        lib().or_mg_eigs(self.h, l, C.byref(a), C.byref(b))
        return a.value, b.value

    def mask(self, l):
        out = np.empty(self.sizes[l])
        lib().or_mg_mask(self.h, l, _p(out))
        return out

    def vcycle(self, r):
        r = _f64(r)
        z = np.zeros_like(r)
        lib().or_mg_vcycle(self.h, _p(r), _p(z))
        return z

    def solve(self, rhs, x0=None, atol=1e-9, rtol=1e-9, max_it=1000):
        rhs = _f64(rhs)
        x = np.zeros_like(rhs) if x0 is None else _f64(x0).copy()
        st = Status()
        lib().or_mg_solve(self.h, _p(rhs), _p(x), atol, rtol, max_it, C.byref(st))
        return x, st.as_dict()


def mprgp_solve(A: Matrix, b, lb, ub, x0=None, atol=1e-9, rtol=1e-9, max_it=1000, eps_eig=1e-1, pm_max_it=10):
    b, lb, ub = _f64(b), _f64(lb), _f64(ub)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    lam = C.c_double()
    lib().or_mprgp_solve(A.h, _p(b), _p(lb), _p(ub), _p(x), atol, rtol, max_it, eps_eig, pm_max_it,
                         C.byref(st), C.byref(lam))
    d = st.as_dict()
    d["lambda_max"] = lam.value
    return x, d


def pgs_solve(A: Matrix, b, lb, ub, x0=None, stol=1e-11, max_it=1000, n_local_sweeps=3, symmetric=True,
              colour=None):
    b, lb, ub = _f64(b), _f64(lb), _f64(ub)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    if colour is not None:
        colour = np.ascontiguousarray(colour, dtype=np.int32)
        nc = int(colour.max()) + 1
        cp = _p(colour)
    else:
        nc, cp = 0, None
    lib().or_pgs_solve(A.h, _p(b), _p(lb), _p(ub), _p(x), stol, max_it, n_local_sweeps, int(symmetric), cp, nc,
                       C.byref(st))
    return x, st.as_dict()


def colouring(A: Matrix):
    out = np.empty(A.nrows, np.int32)
    nc = lib().or_colouring(A.h, _p(out))
    return out, nc


def projected_gradient_norm(A: Matrix, b, lb, ub, x) -> float:
    b, lb, ub, x = _f64(b), _f64(lb), _f64(ub), _f64(x)
    return lib().or_projected_gradient_norm(A.h, _p(b), _p(lb), _p(ub), _p(x))


def edge_grad(src, dst, theta, lam, x):
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    theta = np.ascontiguousarray(theta, np.float32)
    lam, x = _f64(lam), _f64(x)
    g = np.empty(src.size)
    lib().or_edge_grad(src.size, _p(src), _p(dst), _p(theta), _p(lam), _p(x), _p(g))
    return g


def pattern_grad(A: Matrix, lam, x):
    lam, x = _f64(lam), _f64(x)
    g = np.empty(A.nnz)
    lib().or_pattern_grad(A.h, _p(lam), _p(x), _p(g))
    return g


def agglomerate(A: Matrix, bmax=3, weight=1.0 / 3, use_additive_correction=False):
    """Agglomerate::create_transfer_matrix: (parent per row, prolongator as an oracle Matrix)."""
    parent = np.empty(A.nrows, np.int32)
    h = lib().or_agglomerate(A.h, int(bmax), float(weight), int(use_additive_correction), _p(parent))
    return parent, Matrix(_handle=h)


def amg_hierarchy(A: Matrix, n_levels=2, bmax=3, weight=1.0 / 3, max_coarse_rows=4096):
    """AlgebraicMultigridBuilder::build: prolongators ordered coarse -> fine (n_levels 0: coarsen
    until at most max_coarse_rows rows) and the aggregation parents, finest first."""
    Ps, parents, cur = [], [], A
    level = 0
    while (n_levels == 0 and (level == 0 or cur.nrows > max_coarse_rows)) or (n_levels and level < n_levels - 1):
        parent, P = agglomerate(cur, bmax, weight)
        if n_levels == 0 and 4 * P.ncols > 3 * cur.nrows:  # coarsening stalled
            break
        Ps.append(P)
        parents.append(parent)
        cur = Matrix(_handle=lib().or_ptap(cur.h, P.h))
        level += 1
    return Ps[::-1], parents


def bicgstab_solve(A: Matrix, b, x0=None, precond="none", mg=None, atol=1e-9, max_it=1000):
    """BiCGStab (utopia_BiCGStab_impl.hpp:44-250); precond "none", "invdiag" or "mg"."""
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    kind = {"none": 0, "invdiag": 1, "mg": 2}[precond]
    lib().or_bicgstab_solve(A.h, _p(b), _p(x), kind, mg.h if mg is not None else None, atol, max_it, C.byref(st))
    return x, st.as_dict()


def ssn_solve(A: Matrix, b, lb=None, ub=None, x0=None, stol=1e-11, max_it=1000, linear_rtol=1e-12):
    """SemismoothNewton (utopia_SemismoothNewton_impl.hpp:74-207) with BiCGStab + InvDiag inner solves;
    returns x, status, and the final active set."""
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    lbp = _p(_f64(lb)) if lb is not None else None
    ubp = _p(_f64(ub)) if ub is not None else None
    keep = (_f64(lb) if lb is not None else None, _f64(ub) if ub is not None else None)
    lbp = _p(keep[0]) if keep[0] is not None else None
    ubp = _p(keep[1]) if keep[1] is not None else None
    st = Status()
    lib().or_ssn_solve(A.h, _p(b), lbp, ubp, _p(x), stol, max_it, linear_rtol, C.byref(st))
    return x, st.as_dict()


def penalty_solve(A: Matrix, b, lb=None, ub=None, x0=None, selection=None, T=None, O=None, S=None,
                  penalty_parameter=1e4, penalty_parameter_max=None, penalty_parameter_factor=1.5, shift=None,
                  stol=1e-11, max_it=1000, linear_rtol=1e-12, linear_max_it=10000):
    """ShiftedPenaltyQPSolver (utopia_ShiftedPenaltyQPSolver_impl.hpp:87-156) with the ShiftedPenalty
    term; CG + InvDiag inner solves.  penalty_parameter_max None: = penalty_parameter (as read()
    sets it).  shift: a constraint-space shift to start from (None: zero, the reset default);
    returns x, status and the final shift."""
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    keep = [None if v is None else _f64(v) for v in (lb, ub, selection)]
    m = b.size  # T and O are square (the transformation maps R^n to R^n)
    sh = np.zeros(m) if shift is None else _f64(shift).copy()
    st = Status()
    pmax = penalty_parameter if penalty_parameter_max is None else penalty_parameter_max
    lbp, ubp, selp = [_p(v) if v is not None else None for v in keep]
    lib().or_penalty_solve(A.h, _p(b), lbp, ubp, _p(x), selp, T.h if T is not None else None, O.h if O is not None else None,
                           S.h if S is not None else None, penalty_parameter, pmax, penalty_parameter_factor,
                           _p(sh), 1 if shift is None else 0, stol, max_it, linear_rtol, linear_max_it,
                           C.byref(st))
    return x, st.as_dict(), sh


def monotone_mg_solve(A: Matrix, b, lb, ub, P_coarse_to_fine, x0=None, colour=None, pre=3, post=3,
                      n_local_sweeps=3, symmetric=True, smoother="chebyshev", omega=1.0, active_tol=0.0,
                      coarse_space_it=1, atol=1e-9, rtol=1e-9, stol=1e-11, max_it=1000):
    """MonotoneMultigrid (utopia_MonotoneMultigrid.hpp:135-319): PGS smoothing on the fine level
    (in the sweep order of `colour`, lexicographic when None), the interpolation of the last
    transfer truncated on the active set, a linear multigrid (fix_semidefinite, no masks) on the
    truncated Galerkin operator.  Returns x, status, the final active set and the last coarse
    operator."""
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    keep = (_f64(lb) if lb is not None else None, _f64(ub) if ub is not None else None)
    lbp = _p(keep[0]) if keep[0] is not None else None
    ubp = _p(keep[1]) if keep[1] is not None else None
    Ps = [p if isinstance(p, Matrix) else Matrix(p) for p in P_coarse_to_fine]
    arr = (C.c_void_p * len(Ps))(*[p.h for p in Ps])
    if colour is not None:
        colour = np.ascontiguousarray(colour, dtype=np.int32)
        nc, cp = int(colour.max()) + 1, _p(colour)
    else:
        nc, cp = 0, None
    st = Status()
    active = np.zeros(b.size, np.int32)
    coarse = C.c_void_p()
    rc = lib().or_mmg_solve(A.h, _p(b), lbp, ubp, _p(x), len(Ps), C.cast(arr, C.c_void_p), cp, nc, pre, post,
                            n_local_sweeps, int(symmetric), SMOOTHERS[smoother], omega, active_tol,
                            coarse_space_it, atol, rtol, stol, max_it, C.byref(st), _p(active), C.byref(coarse))
    if rc < 0:
        raise RuntimeError("oracle monotone multigrid: coarse operator not SPD")
    return x, st.as_dict(), active, Matrix(_handle=coarse.value)
