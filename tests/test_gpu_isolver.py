"""The isolver plugin (include/isolver_lsolve.h) called the way an external code calls utopia's
plugin: host CRS arrays and vectors through the ten isolver_lsolve_* entry points of libugpu.
The solution is checked against the oracle's Jacobi-preconditioned CG on the same matrix."""
import ctypes as C

import numpy as np
import pytest

import utopia_gb300 as U  # noqa: F401  (loads the library with its signatures)
from utopia_gb300 import _abi
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def test_isolver_plugin_solves_and_refreshes_values(oracle):
    lib = _abi.load()
    A = P.lognormal_diffusion_3d(24, 7)[0]
    n = A.nrows
    rp = np.ascontiguousarray(A.rowptr, np.int32)
    ci = np.ascontiguousarray(A.colidx, np.int32)
    vals = np.ascontiguousarray(A.values, np.float64).copy()
    b = np.random.default_rng(3).uniform(-1, 1, n)
    atol = 1e-10 * np.linalg.norm(b)
    info = _abi.IsolverLsolve()
    assert lib.isolver_lsolve_init(C.byref(info)) == 0 and info.private_data
    try:
        assert lib.isolver_lsolve_set_atol(C.byref(info), atol) == 0
        assert lib.isolver_lsolve_set_max_iterations(C.byref(info), 3000) == 0
        assert lib.isolver_lsolve_set_rtol(C.byref(info), 1e-12) == 0
        assert lib.isolver_lsolve_set_stol(C.byref(info), 1e-14) == 0
        assert lib.isolver_lsolve_set_verbosity(C.byref(info), 0) == 0
        assert lib.isolver_lsolve_update_crs(C.byref(info), n, n, _p(rp, C.c_int), _p(ci, C.c_int),
                                             _p(vals, C.c_double)) == 0
        x = np.zeros(n)
        assert lib.isolver_lsolve_apply(C.byref(info), _p(b, C.c_double), _p(x, C.c_double)) == 0
        xr, st = oracle.cg_solve(oracle.Matrix(A), b, precond="invdiag", atol=atol, max_it=3000)
        assert st["converged"]
        assert np.linalg.norm(b - A.matvec(x)) <= atol * 1.0001
        assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)

        # same pattern arrays, new values: a value refresh; 2A x = b gives x / 2
        vals *= 2.0
        assert lib.isolver_lsolve_update_crs(C.byref(info), n, n, _p(rp, C.c_int), _p(ci, C.c_int),
                                             _p(vals, C.c_double)) == 0
        x2 = np.zeros(n)
        assert lib.isolver_lsolve_apply(C.byref(info), _p(b, C.c_double), _p(x2, C.c_double)) == 0
        assert np.linalg.norm(x2 - 0.5 * xr) <= 1e-8 * np.linalg.norm(xr)

        # a separate preconditioner matrix (here the operator's diagonal): the Jacobi
        # preconditioner takes its diagonal from it; the warm start x2 is kept
        d = A.to_scipy().diagonal() * 2.0
        prp = np.arange(n + 1, dtype=np.int32)
        pci = np.arange(n, dtype=np.int32)
        assert lib.isolver_lsolve_update_with_preconditioner_crs(
            C.byref(info), n, n, _p(rp, C.c_int), _p(ci, C.c_int), _p(vals, C.c_double), _p(prp, C.c_int),
            _p(pci, C.c_int), _p(d, C.c_double)) == 0
        assert lib.isolver_lsolve_apply(C.byref(info), _p(b, C.c_double), _p(x2, C.c_double)) == 0
        assert np.linalg.norm(b - 2.0 * A.matvec(x2)) <= atol * 1.0001

        # distributed sizes are not served by the single-GPU plugin
        assert lib.isolver_lsolve_update_crs(C.byref(info), n // 2, n, _p(rp, C.c_int), _p(ci, C.c_int),
                                             _p(vals, C.c_double)) < 0
    finally:
        assert lib.isolver_lsolve_destroy(C.byref(info)) == 0
    assert not info.private_data
