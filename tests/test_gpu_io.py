"""PETSc binary and raw CRS files through the C ABI, and the ls_solve app on the reference's own
Laplace input (utopia/data/laplace/matrices_for_petsc, decoded into tests/golden/laplace_hierarchy.npz)."""
import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import ls_solve
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def petsc_mat_bytes(A: P.CSR) -> bytes:
    """PETSc binary matrix: big-endian int32 classid 1211216, M, N, nnz, row lengths, columns,
    float64 values."""
    head = np.array([1211216, A.nrows, A.ncols, A.nnz], ">i4").tobytes()
    return (head + np.diff(A.rowptr).astype(">i4").tobytes() + np.asarray(A.colidx, ">i4").tobytes()
            + np.asarray(A.values, ">f8").tobytes())


def petsc_vec_bytes(v) -> bytes:
    return np.array([1211214, v.size], ">i4").tobytes() + np.asarray(v, ">f8").tobytes()


def test_petsc_binary_round_trip(ctx, laplace_hierarchy, tmp_path):
    A, _, rhs = laplace_hierarchy
    rhs = np.asarray(rhs, np.float64)
    fa, fb = tmp_path / "A.bin", tmp_path / "rhs.bin"
    fa.write_bytes(petsc_mat_bytes(A))
    fb.write_bytes(petsc_vec_bytes(rhs))
    M = U.read_petsc_matrix(ctx, fa)
    rp, ci, v = M.csr()
    assert M.shape == (A.nrows, A.ncols)
    np.testing.assert_array_equal(rp, A.rowptr)
    np.testing.assert_array_equal(ci, A.colidx)
    np.testing.assert_array_equal(v, A.values)
    b = U.read_petsc_vector(ctx, fb)
    np.testing.assert_array_equal(b.numpy(), rhs)
    M.write_petsc(tmp_path / "A2.bin")
    b.write_petsc(tmp_path / "rhs2.bin")
    assert (tmp_path / "A2.bin").read_bytes() == fa.read_bytes()
    assert (tmp_path / "rhs2.bin").read_bytes() == fb.read_bytes()


def test_file_errors_are_codes(ctx, tmp_path):
    bad = tmp_path / "bad.bin"
    bad.write_bytes(np.array([1211214, 3], ">i4").tobytes() + b"\0" * 24)  # a vector, read as a matrix
    with pytest.raises(U.UgpuError) as e:
        U.read_petsc_matrix(ctx, bad)
    assert e.value.code == -2
    short = tmp_path / "short.bin"
    short.write_bytes(np.array([1211214, 10], ">i4").tobytes() + b"\0" * 8)
    with pytest.raises(U.UgpuError):
        U.read_petsc_vector(ctx, short)
    with pytest.raises(U.UgpuError):
        U.read_petsc_vector(ctx, tmp_path / "missing.bin")


@pytest.mark.parametrize("ib,vb", [(4, 8), (8, 4)])
def test_raw_crs_round_trip(ctx, tmp_path, ib, vb):
    A = P.lognormal_diffusion_3d(10, 2)[0]
    it = np.int32 if ib == 4 else np.int64
    vt = np.float64 if vb == 8 else np.float32
    np.asarray(A.rowptr, it).tofile(tmp_path / "rowptr.raw")
    np.asarray(A.colidx, it).tofile(tmp_path / "colidx.raw")
    np.asarray(A.values, vt).tofile(tmp_path / "values.raw")
    x = np.random.default_rng(1).standard_normal(A.nrows)
    np.asarray(x, vt).tofile(tmp_path / "x.raw")
    M = U.read_raw_crs(ctx, tmp_path, ib, vb)
    rp, ci, v = M.csr()
    np.testing.assert_array_equal(rp, A.rowptr)
    np.testing.assert_array_equal(ci, A.colidx)
    np.testing.assert_array_equal(v, np.asarray(A.values, vt).astype(np.float64))
    xv = U.read_raw_vector(ctx, tmp_path / "x.raw", vb)
    np.testing.assert_array_equal(xv.numpy(), np.asarray(x, vt).astype(np.float64))
    xv.write_raw(tmp_path / "x64.raw")
    np.testing.assert_array_equal(np.fromfile(tmp_path / "x64.raw", np.float64), xv.numpy())


def test_ls_solve_on_the_reference_laplace_input(ctx, laplace_hierarchy, tmp_path, oracle):
    A, _, rhs = laplace_hierarchy
    rhs = np.asarray(rhs, np.float64)
    (tmp_path / "A.bin").write_bytes(petsc_mat_bytes(A))
    (tmp_path / "rhs.bin").write_bytes(petsc_vec_bytes(rhs))
    xo, st = oracle.cg_solve(oracle.Matrix(A), rhs, precond="invdiag", atol=1e-12, max_it=5000)
    (tmp_path / "x_oracle.bin").write_bytes(petsc_vec_bytes(xo))
    for extra in ([], ["--use_amg"], ["--use_amg", "--amg_as_preconditioner", "0", "--max_it", "500"]):
        out = ls_solve.main(["-A", str(tmp_path / "A.bin"), "-b", str(tmp_path / "rhs.bin"), "--atol", "1e-10",
                             "--oracle", str(tmp_path / "x_oracle.bin"), "--out", str(tmp_path / "x.bin")] + extra)
        assert out["converged"], (extra, out)
        assert out["residual_norm"] <= 1e-10 * 1.0001
        assert out["error_vs_oracle"] < 1e-6
        x = U.read_petsc_vector(ctx, tmp_path / "x.bin").numpy()
        assert np.linalg.norm(rhs - A.matvec(x)) <= 1e-10 * 1.0001
    # raw CRS input (directory) gives the same solve
    np.asarray(A.rowptr, np.int32).tofile(tmp_path / "rowptr.raw")
    np.asarray(A.colidx, np.int32).tofile(tmp_path / "colidx.raw")
    np.asarray(A.values, np.float64).tofile(tmp_path / "values.raw")
    rhs.tofile(tmp_path / "rhs.raw")
    out = ls_solve.main(["-A", str(tmp_path / "rowptr.raw"), "-b", str(tmp_path / "rhs.raw"), "--atol", "1e-10",
                         "--out", str(tmp_path / "x.raw")])
    assert out["converged"] and out["residual_norm"] <= 1e-10 * 1.0001
