"""The reference's own solver templates, compiled here from the reference checkout over a
CPU CSR backend (oracle/ref/*) -- TEST INFRASTRUCTURE ONLY: it pins the restated oracle.

``build_ref(reference_dir)`` compiles ``oracle/ref/ref_solvers.cpp`` together with the
reference's headers and the few support sources its solvers link against (input/config
plumbing, logging, timing) straight from the checkout with g++, into
``oracle/_ref/libutopia_ref.so``.  No reference source is copied into this repository;
the configuration header the reference's CMake would generate is replaced by
``oracle/ref/config/``, which enables no optional backend.

The Python functions mirror the restated oracle's (``oracle.cg_solve``, ``oracle.Multigrid``,
``oracle.mprgp_solve``, ``oracle.pgs_solve``) so that a test runs both on the same input.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(_HERE, "_ref")
_SO = os.path.join(_OUT, "libutopia_ref.so")
_SRC = os.path.join(_HERE, "ref", "ref_solvers.cpp")
_DEPS = [os.path.join(_HERE, "ref", f) for f in ("utopia_ref_backend.hpp", "ref_solvers.cpp")] + [
    os.path.join(_HERE, "ref", "config", f) for f in ("utopia_Config.hpp", "utopia_Version.hpp")]
DEFAULT_REFERENCE = os.environ.get("UTOPIA_REFERENCE_DIR", "/root/reference")

# support sources of the reference (paths inside utopia/) that the solver templates link against
SUPPORT_SOURCES = [
    "utopia_Instance.cpp", "ui/utopia_Input.cpp", "ui/utopia_InputParameters.cpp", "ui/utopia_Banner.cpp",
    "ui/utopia_ui.cpp", "ui/utopia_XMLInput.cpp", "ui/utopia_JSONInput.cpp", "utils/utopia_Chrono.cpp",
    "utils/utopia_Path.cpp", "utils/utopia_MPI.cpp", "utils/utopia_CSV.cpp", "utils/utopia_CiteUtopia.cpp",
    "utils/utopia_AuthoredWork.cpp", "utils/utopia_Utils.cpp", "utopia_core/console/utopia_Reporter.cpp",
    "utopia_core/console/utopia_Logger.cpp", "utopia_core/utopia_Tracer.cpp",
    "utopia_core/interfaces/utopia_Communicator.cpp", "utopia_core/utopia_BackendInfo.cpp",
]
_MODULES = ["utopia_core", "solvers", "utils", "ui", "interoperability", "differentiable", "backend/polymorphic"]

_lock = threading.Lock()
_lib = None


def reference_available(reference_dir: str = DEFAULT_REFERENCE) -> bool:
    return os.path.isdir(os.path.join(reference_dir, "utopia", "solvers"))


def _include_flags(reference_dir):
    root = os.path.join(reference_dir, "utopia")
    dirs = [os.path.join(_HERE, "ref", "config"), os.path.join(_HERE, "ref"), root]
    for m in _MODULES:
        for d, sub, _ in os.walk(os.path.join(root, m)):
            sub[:] = sorted(s for s in sub if s not in ("rapidjson", "rapidxml", "windows"))
            dirs.append(d)
    dirs += [os.path.join(root, "ui", "rapidxml"), os.path.join(root, "ui", "rapidjson", "include")]
    out = []
    for d in dirs:
        out += ["-I", d]
    return out


def build_ref(reference_dir: str = DEFAULT_REFERENCE, force: bool = False) -> str | None:
    """Compile oracle/_ref/libutopia_ref.so from the reference checkout (None if it is absent)."""
    if not reference_available(reference_dir):
        return None
    newest = max(os.path.getmtime(p) for p in _DEPS)
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= newest:
        return _SO
    os.makedirs(os.path.join(_OUT, "obj"), exist_ok=True)
    inc = _include_flags(reference_dir)
    base = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-w"]
    root = os.path.join(reference_dir, "utopia")

    def compile_one(src):
        obj = os.path.join(_OUT, "obj", os.path.basename(src) + ".o")
        subprocess.run(base + inc + ["-c", src, "-o", obj], check=True, capture_output=True, text=True)
        return obj

    srcs = [_SRC] + [os.path.join(root, s) for s in SUPPORT_SOURCES]
    try:
        with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
            objs = list(ex.map(compile_one, srcs))
    except subprocess.CalledProcessError as e:
        raise RuntimeError(f"building the reference oracle failed:\n{e.stderr[-4000:]}") from e
    subprocess.run(["g++", "-shared", "-o", _SO + ".tmp", *objs, "-Wl,--no-undefined"], check=True)
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


_vp, _d, _i64, _i32 = C.c_void_p, C.c_double, C.c_int64, C.c_int32


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_SO):
                raise RuntimeError("oracle/_ref/libutopia_ref.so is not built (the reference checkout is needed)")
            L = C.CDLL(_SO)
            sig = {
                "ref_csr_create": (_vp, [_i64, _i64, _vp, _vp, _vp]),
                "ref_csr_free": (None, [_vp]),
                "ref_csr_nnz": (_i64, [_vp]),
                "ref_csr_rows": (_i64, [_vp]),
                "ref_csr_arrays": (None, [_vp, _vp, _vp, _vp]),
                "ref_mg_create": (_vp, [_vp, _i32, _vp, _i32, _i32, _i32, _i32]),
                "ref_mg_free": (None, [_vp]),
                "ref_mg_levels": (_i32, [_vp]),
                "ref_mg_level_matrix": (_vp, [_vp, _i32]),
                "ref_mg_solve": (_i32, [_vp, _vp, _vp, _d, _d, _i64, _vp]),
                "ref_cg_solve": (_i32, [_vp, _vp, _vp, _i32, _vp, _d, _d, _d, _i64, _vp]),
                "ref_mprgp_solve": (_i32, [_vp, _vp, _vp, _vp, _vp, _d, _d, _i64, _vp]),
                "ref_pgs_solve": (_i32, [_vp, _vp, _vp, _vp, _vp, _d, _i64, _i32, _i32, _vp]),
                "ref_penalty_solve": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _i32, _i32,
                                             _d, _i64, _d, _i64, _vp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _csr_arrays(h):
    n = lib().ref_csr_rows(h)
    nnz = lib().ref_csr_nnz(h)
    rp, ci, v = np.empty(n + 1, np.int32), np.empty(nnz, np.int32), np.empty(nnz)
    lib().ref_csr_arrays(h, _p(rp), _p(ci), _p(v))
    return rp, ci, v


class Matrix:
    """A CSR matrix of the reference backend (copied from a problems.CSR)."""

    def __init__(self, csr):
        self.nrows, self.ncols = int(csr.nrows), int(csr.ncols)
        rp = np.ascontiguousarray(csr.rowptr, np.int32)
        ci = np.ascontiguousarray(csr.colidx, np.int32)
        v = _f64(csr.values)
        self.h = lib().ref_csr_create(self.nrows, self.ncols, _p(rp), _p(ci), _p(v))

    def __del__(self):
        try:
            lib().ref_csr_free(self.h)
        except Exception:
            pass

    def arrays(self):
        return _csr_arrays(self.h)


SMOOTHERS = {"jacobi": 0, "chebyshev": 1, "point_jacobi": 2}


class Multigrid:
    """utopia::Multigrid<Matrix, Vector> (V-cycle, IPRTransfer, Galerkin RAP, masks, dense
    Cholesky coarse solve) over the reference backend."""

    def __init__(self, A: Matrix, P_coarse_to_fine, smoother="chebyshev", pre=3, post=3, fix_semidefinite=False):
        self._P = [p if isinstance(p, Matrix) else Matrix(p) for p in P_coarse_to_fine]
        arr = (C.c_void_p * len(self._P))(*[p.h for p in self._P])
        self.h = lib().ref_mg_create(A.h, len(self._P), C.cast(arr, C.c_void_p), SMOOTHERS[smoother], pre, post,
                                     int(fix_semidefinite))
        if not self.h:
            raise RuntimeError("reference multigrid set-up failed")
        self.n_levels = lib().ref_mg_levels(self.h)

    def __del__(self):
        try:
            lib().ref_mg_free(self.h)
        except Exception:
            pass

    def level_matrix_arrays(self, l):
        return _csr_arrays(lib().ref_mg_level_matrix(self.h, l))

    def solve(self, rhs, x0=None, atol=1e-9, rtol=1e-9, max_it=1000):
        rhs = _f64(rhs)
        x = np.zeros_like(rhs) if x0 is None else _f64(x0).copy()
        st = Status()
        if lib().ref_mg_solve(self.h, _p(rhs), _p(x), atol, rtol, max_it, C.byref(st)) != 0:
            raise RuntimeError("reference multigrid solve failed")
        return x, st.as_dict()


def cg_solve(A: Matrix, b, x0=None, precond="invdiag", mg=None, atol=1e-9, rtol=1e-9, stol=1e-11, max_it=1000):
    b = _f64(b)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    code = {"none": 0, "invdiag": 1, "mg": 2}[precond]
    if lib().ref_cg_solve(A.h, _p(b), _p(x), code, mg.h if mg is not None else None, atol, rtol, stol, max_it,
                          C.byref(st)) != 0:
        raise RuntimeError("reference CG failed")
    return x, st.as_dict()


def mprgp_solve(A: Matrix, b, lb, ub, x0=None, atol=1e-9, rtol=1e-9, max_it=1000):
    b = _f64(b)
    lb = None if lb is None else _f64(lb)
    ub = None if ub is None else _f64(ub)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    if lib().ref_mprgp_solve(A.h, _p(b), _p(lb), _p(ub), _p(x), atol, rtol, max_it, C.byref(st)) != 0:
        raise RuntimeError("reference MPRGP failed")
    return x, st.as_dict()


def pgs_solve(A: Matrix, b, lb, ub, x0=None, stol=1e-11, max_it=1000, n_local_sweeps=3, symmetric=True):
    b = _f64(b)
    lb = None if lb is None else _f64(lb)
    ub = None if ub is None else _f64(ub)
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    if lib().ref_pgs_solve(A.h, _p(b), _p(lb), _p(ub), _p(x), stol, max_it, n_local_sweeps, int(symmetric),
                           C.byref(st)) != 0:
        raise RuntimeError("reference projected Gauss-Seidel failed")
    return x, st.as_dict()


def penalty_solve(A: Matrix, b, lb=None, ub=None, x0=None, selection=None, T=None, O=None, S=None,
                  penalty_parameter=1e4, penalty_parameter_max=None, penalty_parameter_factor=1.5,
                  zero_shift_on_reset=True, n_solves=1, stol=1e-11, max_it=1000, linear_rtol=1e-12,
                  linear_max_it=10000):
    """The reference's ShiftedPenaltyQPSolver (CG + InvDiag inner solves to linear_rtol ||rhs||);
    n_solves consecutive solves by one solver object, each from the previous x."""
    b = _f64(b)
    lb, ub, selection = (None if v is None else _f64(v) for v in (lb, ub, selection))
    x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
    st = Status()
    pmax = penalty_parameter if penalty_parameter_max is None else penalty_parameter_max
    rc = lib().ref_penalty_solve(A.h, _p(b), _p(lb), _p(ub), _p(x), _p(selection),
                                 T.h if T is not None else None, O.h if O is not None else None,
                                 S.h if S is not None else None, penalty_parameter, pmax, penalty_parameter_factor,
                                 int(bool(zero_shift_on_reset)), int(n_solves), stol, max_it, linear_rtol,
                                 linear_max_it, C.byref(st))
    if rc != 0:
        raise RuntimeError("reference shifted-penalty solver failed")
    return x, st.as_dict()
