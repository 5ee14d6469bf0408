"""CPU checks of the C-ABI library: it builds, loads without a GPU, exports every entry
point declared in include/ugpu.h and include/isolver_lsolve.h, and reports a missing device
as an error code."""
import ctypes
import os
import subprocess

import pytest

from utopia_gb300 import _abi


@pytest.fixture(scope="module")
def lib():
    from utopia_gb300 import build

    build.build()
    return _abi.load()


def test_header_declares_the_boundary():
    syms = _abi.header_symbols()
    for s in ("ugpu_create", "ugpu_spmv", "ugpu_ptap", "ugpu_solver_apply", "ugpu_mg_set_transfer_operators",
              "ugpu_qp_set_box_constraints", "ugpu_residual", "ugpu_dots"):
        assert s in syms
    assert set(_abi.SIGNATURES) == set(syms), "ctypes signatures and the header disagree"


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in _abi.header_symbols() if s not in exported]
    assert not missing, missing
    for s in _abi.header_symbols():
        assert hasattr(lib, s)


def test_library_is_built_for_sm_103a():
    # the fat binary carries sm_103a code (inspected through the compiler's own listing tool is
    # not needed: the build command pins -gencode arch=compute_103a,code=sm_103a)
    from utopia_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_device_is_an_error_code_not_a_crash(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.ugpu_create(0, ctypes.byref(h))
    assert rc < 0
    assert lib.ugpu_last_error(None)


def test_null_handles_are_rejected(lib):
    assert lib.ugpu_spmv(None, None, None) == -2
    assert lib.ugpu_solver_apply(None, None, None) == -2
    assert lib.ugpu_vec_destroy(None) == 0


def test_isolver_plugin_is_exported(lib):
    """The ten isolver_lsolve_* entry points of utopia's isolver plugin are served by libugpu."""
    syms = _abi.isolver_symbols()
    assert len(syms) == 10 and set(syms) == set(_abi.ISOLVER_SIGNATURES)
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert not [s for s in syms if s not in exported]


def test_isolver_plugin_errors_without_state(lib):
    import torch

    assert lib.isolver_lsolve_init(None) == -2
    info = _abi.IsolverLsolve()
    x = (ctypes.c_double * 4)()
    assert lib.isolver_lsolve_apply(ctypes.byref(info), x, x) == -5  # no solver in private_data
    assert lib.isolver_lsolve_set_atol(ctypes.byref(info), 1e-9) == -5
    assert lib.isolver_lsolve_destroy(ctypes.byref(info)) == 0
    if not torch.cuda.is_available():
        assert lib.isolver_lsolve_init(ctypes.byref(info)) < 0 and not info.private_data
