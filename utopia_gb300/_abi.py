"""ctypes binding of libugpu (include/ugpu.h).

The shared library is built in-tree by ``utopia_gb300.build``; this module never
falls back to anything else: if the library or a GPU is missing, calls raise.
"""

from __future__ import annotations

import ctypes as C
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libugpu.so")
HEADER = os.path.join(ROOT, "include", "ugpu.h")

F64, F32, BF16 = 0, 1, 2
FORMAT_CSR, FORMAT_SELL = 0, 1
SOLVER_CG, SOLVER_MULTIGRID, SOLVER_INVDIAG, SOLVER_MPRGP, SOLVER_PGS, SOLVER_CHOLESKY = 1, 2, 3, 4, 5, 6
SOLVER_AMG = 7
SOLVER_BICGSTAB = 8
SOLVER_SSNEWTON = 9
SOLVER_MONOTONE_MG = 10
SOLVER_SHIFTED_PENALTY = 11

_lock = threading.Lock()
_lib = None


class UgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ugpu error {code}: {msg}")
        self.code = code


class SolutionStatus(C.Structure):
    _fields_ = [
        ("iterates", C.c_int64),
        ("gradient_norm", C.c_double),
        ("relative_gradient_norm", C.c_double),
        ("step_norm", C.c_double),
        ("reason", C.c_int32),
        ("converged", C.c_int32),
        ("spmv_count", C.c_int64),
        ("execution_time", C.c_double),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_vp, _d, _i64, _i32, _int = C.c_void_p, C.c_double, C.c_int64, C.c_int32, C.c_int
_pp = C.POINTER(C.c_void_p)

SIGNATURES = {
    "ugpu_create": [_int, _pp],
    "ugpu_destroy": [_vp],
    "ugpu_last_error": [_vp],
    "ugpu_synchronize": [_vp],
    "ugpu_launch_count": [_vp, C.POINTER(_i64)],
    "ugpu_stream": [_vp, _pp],
    "ugpu_vec_create": [_vp, _i64, _int, _pp],
    "ugpu_vec_wrap_device": [_vp, _vp, _i64, _int, _pp],
    "ugpu_vec_destroy": [_vp],
    "ugpu_vec_size": [_vp, C.POINTER(_i64), C.POINTER(_int)],
    "ugpu_vec_device_ptr": [_vp, _pp],
    "ugpu_vec_upload": [_vp, _vp],
    "ugpu_vec_download": [_vp, _vp],
    "ugpu_vec_set": [_vp, _d],
    "ugpu_vec_copy": [_vp, _vp],
    "ugpu_axpby": [_d, _vp, _d, _vp],
    "ugpu_dot": [_vp, _vp, C.POINTER(_d)],
    "ugpu_dots": [_int, _pp, _pp, C.POINTER(_d)],
    "ugpu_norm2": [_vp, C.POINTER(_d)],
    "ugpu_pointwise": [_int, _vp, _vp, _vp],
    "ugpu_pseudo_inverse": [_vp, _vp, _d],
    "ugpu_multi_min": [_vp, _vp, C.POINTER(_d)],
    "ugpu_vec_reduce": [_vp, _i32, C.POINTER(_d)],
    "ugpu_vec_transform": [_vp, _i32, _d],
    "ugpu_active_set_compact": [_vp, _vp, _vp, _i32, _vp, C.POINTER(_i64)],
    "ugpu_test_staged_wait_timeout": [_vp, _vp, _vp, _i64, C.POINTER(_int)],
    "ugpu_dots_noalloc": [_int, _pp, _pp, C.POINTER(_int), C.POINTER(_int), _i64, _vp, _vp],
    "ugpu_csr_create": [_vp, _i64, _i64, _i64, _vp, _vp, _vp, _pp],
    "ugpu_csr_create_device": [_vp, _i64, _i64, _i64, _vp, _vp, _vp, _pp],
    "ugpu_mat_destroy": [_vp],
    "ugpu_mat_info": [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_int)],
    "ugpu_csr_download": [_vp, _vp, _vp, _vp],
    "ugpu_mat_update_values": [_vp, _vp],
    "ugpu_mat_cast": [_vp, _int, _pp],
    "ugpu_mat_set_format": [_vp, _int],
    "ugpu_mat_sell_info": [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_int)],
    "ugpu_mat_sell_layout": [_vp, C.POINTER(_int), C.POINTER(_i64)],
    "ugpu_diag": [_vp, _vp],
    "ugpu_transpose": [_vp, _pp],
    "ugpu_spgemm": [_vp, _vp, _pp],
    "ugpu_ptap": [_vp, _vp, _pp],
    "ugpu_ptap_reuse": [_vp, _vp, _int, _pp],
    "ugpu_spmv": [_vp, _vp, _vp],
    "ugpu_spmv_add": [_vp, _vp, _vp, _vp],
    "ugpu_fp64_rate": [_vp, _int, C.POINTER(C.c_double)],
    "ugpu_spmv_dot": [_vp, _vp, _vp, _vp],
    "ugpu_residual": [_vp, _vp, _vp, _vp],
    "ugpu_jacobi_sweep": [_vp, _vp, _vp, _d, _vp],
    "ugpu_solver_create": [_vp, _int, _pp],
    "ugpu_solver_destroy": [_vp],
    "ugpu_solver_set": [_vp, C.c_char_p, _d],
    "ugpu_solver_get": [_vp, C.c_char_p, C.POINTER(_d)],
    "ugpu_solver_set_preconditioner": [_vp, _vp],
    "ugpu_mg_set_transfer_operators": [_vp, _int, _pp],
    "ugpu_mg_level_matrix": [_vp, _int, _pp],
    "ugpu_mg_n_levels": [_vp, C.POINTER(_int)],
    "ugpu_mg_eigs": [_vp, _int, C.POINTER(_d), C.POINTER(_d)],
    "ugpu_mg_vcycle": [_vp, _vp, _vp],
    "ugpu_solver_update": [_vp, _vp],
    "ugpu_solver_apply": [_vp, _vp, _vp],
    "ugpu_solver_solve": [_vp, _vp, _vp, _vp],
    "ugpu_qp_set_box_constraints": [_vp, _vp, _vp],
    "ugpu_solver_status": [_vp, C.POINTER(SolutionStatus)],
    "ugpu_project": [_vp, _vp, _vp],
    "ugpu_pgs_colouring": [_vp, _vp, C.POINTER(_int)],
    "ugpu_amg_parent": [_vp, _int, _vp, C.POINTER(_i64), C.POINTER(_i64)],
    "ugpu_mmg_active_set": [_vp, _vp, C.POINTER(_i64)],
    "ugpu_penalty_set_transform": [_vp, _vp, _vp],
    "ugpu_penalty_set_selection": [_vp, _vp],
    "ugpu_penalty_set_scaling_matrix": [_vp, _vp],
    "ugpu_petsc_read_mat": [_vp, C.c_char_p, _pp],
    "ugpu_petsc_read_vec": [_vp, C.c_char_p, _pp],
    "ugpu_petsc_write_mat": [_vp, C.c_char_p],
    "ugpu_petsc_write_vec": [_vp, C.c_char_p],
    "ugpu_raw_crs_read": [_vp, C.c_char_p, _int, _int, _i64, _pp],
    "ugpu_raw_vec_read": [_vp, C.c_char_p, _int, _pp],
    "ugpu_raw_vec_write": [_vp, C.c_char_p],
    "ugpu_graph_create": [_vp, _i64, _i64, _vp, _vp, _i64, _vp, _vp, _pp],
    "ugpu_graph_destroy": [_vp],
    "ugpu_graph_assemble": [_vp, _vp, _vp],
    "ugpu_graph_edge_grad": [_vp, _vp, _vp, _vp, _vp],
    "ugpu_pattern_grad": [_vp, _vp, _vp, _vp],
}


ISOLVER_HEADER = os.path.join(os.path.dirname(HEADER), "isolver_lsolve.h")


class IsolverLsolve(C.Structure):
    """isolver_lsolve_t: communicator slot and the solver's private data."""

    _fields_ = [("comm", C.c_void_p), ("private_data", C.c_void_p)]


_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_info = C.POINTER(IsolverLsolve)
ISOLVER_SIGNATURES = {
    "isolver_lsolve_init": [_info],
    "isolver_lsolve_update_crs": [_info, C.c_ssize_t, C.c_ssize_t, _ip, _ip, _dp],
    "isolver_lsolve_update_with_preconditioner_crs": [_info, C.c_ssize_t, C.c_ssize_t, _ip, _ip, _dp, _ip, _ip,
                                                      _dp],
    "isolver_lsolve_apply": [_info, _dp, _dp],
    "isolver_lsolve_set_max_iterations": [_info, C.c_int],
    "isolver_lsolve_set_atol": [_info, C.c_double],
    "isolver_lsolve_set_stol": [_info, C.c_double],
    "isolver_lsolve_set_rtol": [_info, C.c_double],
    "isolver_lsolve_set_verbosity": [_info, C.c_int],
    "isolver_lsolve_destroy": [_info],
}


def isolver_symbols(path: str = ISOLVER_HEADER):
    """Function names declared with ISOLVER_EXPORT in include/isolver_lsolve.h."""
    txt = open(path).read()
    return sorted(set(re.findall(r"ISOLVER_EXPORT\s+(isolver_\w+)\s*\(", txt)))


def header_symbols(path: str = HEADER):
    """Function names declared with UGPU_API in include/ugpu.h."""
    txt = open(path).read()
    return sorted(set(re.findall(r"UGPU_API\s+[\w\s\*]+?\b(ugpu_\w+)\s*\(", txt)))


def load(path: str = LIB_PATH):
    """Load libugpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(f"libugpu.so is not built ({path}); run __graft_entry__.build()")
            L = C.CDLL(path)
            for name, args in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = C.c_char_p if name == "ugpu_last_error" else C.c_int
            for name, args in ISOLVER_SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = C.c_int
            _lib = L
    return _lib


def check(rc: int, ctx=None):
    if rc != 0:
        msg = load().ugpu_last_error(ctx)
        raise UgpuError(rc, msg.decode() if msg else "")
