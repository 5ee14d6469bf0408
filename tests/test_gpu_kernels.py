"""GPU parity of the BLAS-1, SpMV-family, transpose and SpGEMM kernels against the oracle,
called through the C ABI."""
import hashlib

import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


def bf16_round(a):
    """Round float64 -> bf16 (nearest even) -> float64, as the storage conversion does."""
    f = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (f >> 16) & 1
    f = ((f + 0x7FFF + lsb) >> 16) << 16
    return f.astype(np.uint32).view(np.float32).astype(np.float64)


def random_csr(n, m, density, seed, long_rows=0):
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    M = sp.random(n, m, density=density, random_state=rng, format="csr")
    if long_rows:
        M = M.tolil()
        for r in rng.choice(n, long_rows, replace=False):
            cols = rng.choice(m, min(m, 700), replace=False)
            M[r, cols] = rng.standard_normal(cols.size)
        M = M.tocsr()
    M.sort_indices()
    return P.CSR.from_scipy(M)


MATRICES = {
    "lap2d": lambda: P.laplacian_2d(70, 33),
    "lap3d": lambda: P.laplacian_3d(20, 19, 18),
    "lognormal": lambda: P.lognormal_diffusion_3d(24, 5)[0],
    "interp": lambda: P.interpolation_3d(16),
    "random": lambda: random_csr(3001, 2777, 0.003, 11),
    "random_long_rows": lambda: random_csr(1500, 1600, 0.004, 12, long_rows=5),
    "empty_rows": lambda: P.CSR(5, 4, np.array([0, 0, 2, 2, 3, 3]), np.array([1, 3, 0]), np.array([1.0, -2.0, 3.0])),
}


def test_vector_roundtrip_and_blas1(ctx):
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(100_003), rng.standard_normal(100_003)
    va, vb = U.Vector(ctx, a), U.Vector(ctx, b)
    np.testing.assert_array_equal(va.numpy(), a)
    d1, d2 = va.dot(vb), va.dot(vb)
    assert d1 == d2  # deterministic reduction order
    assert abs(d1 - a @ b) <= 1e-12 * np.abs(a * b).sum()
    assert abs(va.norm2() - np.linalg.norm(a)) <= 1e-13 * np.linalg.norm(a)
    vb.axpby(2.0, va, -0.5)
    np.testing.assert_allclose(vb.numpy(), 2 * a - 0.5 * b, rtol=1e-15, atol=1e-15)
    out = U.dots([(va, va), (va, vb)])
    assert abs(out[0] - a @ a) <= 1e-12 * (a @ a)
    v32 = U.Vector(ctx, n=a.size, dtype=U.F32)
    va.copy_to(v32)
    np.testing.assert_array_equal(v32.numpy(), a.astype(np.float32))


@pytest.mark.parametrize("offset", [0, 1, 2])
def test_pinned_host_upload_download(ctx, offset):
    """Pinned host buffers, aligned or not, and pageable ones give the same bytes both ways."""
    torch = pytest.importorskip("torch")
    n = 300_001
    a = np.random.default_rng(offset).standard_normal(n + 2)
    hb = torch.from_numpy(a).pin_memory()
    hx = torch.full((n + 2,), -1.0, dtype=torch.float64).pin_memory()
    v = U.Vector(ctx, n=n)
    v.upload_from(hb.data_ptr() + 8 * offset)
    np.testing.assert_array_equal(v.numpy(), a[offset:offset + n])
    v.download_to(hx.data_ptr() + 8 * offset)
    h = hx.numpy()
    np.testing.assert_array_equal(h[offset:offset + n], a[offset:offset + n])
    assert np.all(h[:offset] == -1.0) and np.all(h[offset + n:] == -1.0)
    page = np.empty(n)
    v.download_to(page.ctypes.data)
    np.testing.assert_array_equal(page, a[offset:offset + n])


def test_fp64_fp32_conversions_match_ieee(ctx):
    """The device converts FP64 <-> FP32 with integer bit operations (round to nearest even);
    results equal numpy's IEEE conversions bit for bit, on ties, the overflow boundary, the
    smallest normals, subnormals (ties included), signed zeros, infinities, NaNs (with their
    payloads) and random magnitudes."""
    rng = np.random.default_rng(7)
    one = 1.0
    edge = [0.0, -0.0, one, -one, one + 2.0**-24, one + 3 * 2.0**-24, one + 2.0**-24 + 2.0**-52,
            np.float32(3.4028235e38).astype(np.float64), 3.4028235677973366e38, 3.4028235677973362e38, 1e39,
            -1e39, 2.0**-126, 2.0**-126 * (1 - 2.0**-25), 2.0**-127, 1e-45, 1e-300, np.inf, -np.inf,
            np.nan, 0.1, 1 / 3, 2.0**-149 * 1.5, 2.0**-150, 2.0**-150 * (1 + 2.0**-52), 3 * 2.0**-150,
            2.0**-149 * 2.5, 2.0**-126 * (1 - 2.0**-24), 2.0**-126 * (1 - 2.0**-23), 5e-324, -5e-324, 2.0**-1022,
            2.0**-149 * 0.5000001, 2.0**-149 * 0.4999999]
    rnd = np.concatenate([rng.standard_normal(20000) * 10.0 ** rng.integers(-40, 40, 20000),
                          rng.uniform(-2.0**-126, 2.0**-126, 20000)])  # the float subnormal range
    d = np.array(edge + list(rnd), dtype=np.float64)
    v64, v32 = U.Vector(ctx, d), U.Vector(ctx, n=d.size, dtype=U.F32)
    v64.copy_to(v32)
    with np.errstate(over="ignore"):
        ref = d.astype(np.float32)
    got = v32.numpy()
    ok = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
    assert ok.all(), d[~ok][:5]
    # NaN payloads: the top fraction bits kept, the quiet bit set (as numpy's conversion does)
    nan64 = np.array([0x7ff8000000000001, 0x7ff0000000000001, 0xfff8123456789abc], np.uint64).view(np.float64)
    n64, n32 = U.Vector(ctx, nan64), U.Vector(ctx, n=3, dtype=U.F32)
    n64.copy_to(n32)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(n32.numpy().view(np.uint32), nan64.astype(np.float32).view(np.uint32))
    f = np.concatenate([ref, np.array([1e-40, -1e-44, 1.17549435e-38], np.float32),
                        (rng.standard_normal(20000) * 10.0 ** rng.integers(-44, 38, 20000)).astype(np.float32)])
    w32, w64 = U.Vector(ctx, f, dtype=U.F32), U.Vector(ctx, n=f.size)
    w32.copy_to(w64)
    got64, ref64 = w64.numpy(), f.astype(np.float64)
    ok = (got64.view(np.uint64) == ref64.view(np.uint64)) | (np.isnan(got64) & np.isnan(ref64))
    assert ok.all(), f[~ok][:5]
    nan32 = np.array([0x7fc00001, 0x7f800001, 0xffc12345], np.uint32).view(np.float32)
    m32, m64 = U.Vector(ctx, nan32, dtype=U.F32), U.Vector(ctx, n=3)
    m32.copy_to(m64)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(m64.numpy().view(np.uint64), nan32.astype(np.float64).view(np.uint64))


def test_empty_vector_dot(ctx):
    v = U.Vector(ctx, n=0)
    assert v.dot(v) == 0.0


@pytest.mark.parametrize("name", list(MATRICES))
def test_spmv_fp64_matches_oracle(ctx, oracle, name):
    A = MATRICES[name]()
    x = np.random.default_rng(1).standard_normal(A.ncols)
    yref = oracle.Matrix(A).matvec(x)
    M = U.SparseMatrix(ctx, A)
    vx, vy = U.Vector(ctx, x), U.Vector(ctx, n=A.nrows)
    bound = 1e-14 * (np.abs(A.to_scipy()) @ np.abs(x)) + 1e-300
    for fmt in (U.FORMAT_SELL, U.FORMAT_CSR):
        M.set_format(fmt)
        M.apply(vx, vy)
        y = vy.numpy()
        assert np.all(np.abs(y - yref) <= 4 * bound), (name, fmt)


@pytest.mark.parametrize("name", ["lap2d", "lap3d", "lognormal"])
def test_spmv_dot_fused(ctx, name):
    """y = A x and (x, y) from one kernel: y bit-identical to the plain product's, the dot within
    1e-13 of numpy's (a different summation order) and identical over repeated calls."""
    A = MATRICES[name]()
    x = np.random.default_rng(2).standard_normal(A.ncols)
    M = U.SparseMatrix(ctx, A)
    vx, vy, vz = U.Vector(ctx, x), U.Vector(ctx, n=A.nrows), U.Vector(ctx, n=A.nrows)
    for fmt in (U.FORMAT_SELL, U.FORMAT_CSR):
        M.set_format(fmt)
        M.apply(vx, vz)
        d = M.apply_dot(vx, vy)
        y = vy.numpy()
        assert np.array_equal(y, vz.numpy()), (name, fmt)
        ref = float(x @ y)
        assert abs(d - ref) <= 1e-13 * (np.abs(x) @ np.abs(y)), (name, fmt)
        assert M.apply_dot(vx, vy) == d


def expected_diagonal_slots(A, S):
    """Stored slots of the diagonal-keyed sliced ELL: per slice of S rows, one slot per
    distinct offset col - row."""
    rows = np.repeat(np.arange(A.nrows), np.diff(A.rowptr))
    off = A.colidx.astype(np.int64) - rows
    total = 0
    for s in range(0, A.nrows, S):
        seg = off[A.rowptr[s]:A.rowptr[min(A.nrows, s + S)]]
        total += np.unique(seg).size * S
    return total


def test_spmv_unaligned_wrapped_input(ctx, oracle):
    """Wrapped caller memory that is not 16-byte aligned is read correctly (CSR path)."""
    A = P.lognormal_diffusion_3d(12, 1)[0]
    x = np.random.default_rng(4).standard_normal(A.ncols)
    big = U.Vector(ctx, np.concatenate([[7.0], x]))  # x starts 8 bytes into the allocation
    vx = U.Vector.wrap_device(ctx, big.device_ptr + 8, A.ncols)
    vy = U.Vector(ctx, n=A.nrows)
    U.SparseMatrix(ctx, A).apply(vx, vy)
    np.testing.assert_allclose(vy.numpy(), oracle.Matrix(A).matvec(x), rtol=1e-13, atol=1e-13)


def torch_sms():
    import torch

    return torch.cuda.get_device_properties(0).multi_processor_count


@pytest.mark.parametrize("dtype", [U.F32, U.BF16])
def test_staged_kernel_matches_register_kernel(ctx, dtype):
    """FP32 / BF16 operators whose slices are all keyed (diagonal: col - row; anchored:
    col - first column of the row) get the lane-interleaved layout and run through the
    shared-memory staged kernel when every vector is 16-byte aligned; a vector 4 bytes into
    its allocation sends the same call to the register kernel.  Both sum each row over the
    same slots in the same order, so the product, residual, add and Jacobi forms agree bit
    for bit: on the 7-point fine operator (24^3 and 48^3), its 27-point Galerkin coarse operator, the
    trilinear interpolation P (anchored, x windows staged) and R = P^T (anchored; its x
    windows are too wide to stage, so both calls take the register kernel).  The transfers are
    taken at 108^3 -> 54^3 so that both have more
    slices than 8 per SM: smaller transfer operators go to the CSR kernel instead of the
    register kernel, which sums in another order."""
    A = P.lognormal_diffusion_3d(24, 5)[0]
    M64 = U.SparseMatrix(ctx, A)
    P24 = U.SparseMatrix(ctx, P.interpolation_3d(24))
    Pcsr = P.interpolation_3d(108)
    Pm = U.SparseMatrix(ctx, Pcsr)
    Rsp = Pcsr.to_scipy().T.tocsr()
    Rsp.sort_indices()
    Rm = U.SparseMatrix(ctx, P.CSR.from_scipy(Rsp))
    assert Rm.sell_info()["nslices"] > 8 * torch_sms()
    rng = np.random.default_rng(11)
    # 48^3: neighbour planes 2304 rows away (their windows staged like the others)
    M48 = U.SparseMatrix(ctx, P.lognormal_diffusion_3d(48, 5)[0])
    for M, square in ((M64, True), (M48, True), (M64.ptap(P24), True), (Pm, False), (Rm, False)):
        Mx = M.cast(dtype)
        assert Mx.sell_interleaved()
        n, m = M.nrows, M.ncols
        x = rng.standard_normal(m).astype(np.float32)
        b, v = (rng.standard_normal(n).astype(np.float32) for _ in range(2))

        def vec(a, aligned):
            if aligned:
                return U.Vector(ctx, a, dtype=U.F32), None
            big = U.Vector(ctx, np.concatenate([[np.float32(3)], a]).astype(np.float32), dtype=U.F32)
            return U.Vector.wrap_device(ctx, big.device_ptr + 4, a.size, U.F32), big

        out = {}
        for aligned in (True, False):
            vx, keep = vec(x, aligned)
            vb, vv = U.Vector(ctx, b, dtype=U.F32), U.Vector(ctx, v, dtype=U.F32)
            ys = [U.Vector(ctx, n=n, dtype=U.F32) for _ in range(4)]
            Mx.apply(vx, ys[0])
            Mx.apply_add(vx, vv, ys[2])
            if square:
                Mx.residual(vb, vx, ys[1])
                Mx.jacobi_sweep(vb, vx, 0.8, ys[3])
            out[aligned] = [y.numpy() for y in ys]
        for a, u in zip(out[True], out[False]):
            assert np.array_equal(a.view(np.uint32), u.view(np.uint32))
        r, c, vals = Mx.csr()
        ref = P.CSR(n, m, r, c, vals).matvec(x.astype(np.float64))
        bound = 1e-6 * (np.abs(P.CSR(n, m, r, c, vals).to_scipy()) @ np.abs(x.astype(np.float64)))
        assert np.all(np.abs(out[True][0] - ref) <= 4 * bound + 1e-30)


def test_transfer_operators_use_anchored_slices(ctx):
    """Rows of the trilinear interpolation and of its transpose share one shape relative to
    their first column: every slice is keyed by col - anchor (no column indices stored), and
    the FP64 products through those slices match scipy."""
    Psp = P.interpolation_3d(24).to_scipy()
    for M in (Psp, Psp.T.tocsr()):
        M.sort_indices()
        C = P.CSR.from_scipy(M)
        Md = U.SparseMatrix(ctx, C)
        info = Md.sell_info()
        assert info["ndiag_slices"] == 0 and Md.sell_anchored_slices() == info["nslices"]
        x = np.random.default_rng(5).standard_normal(C.ncols)
        y = U.Vector(ctx, n=C.nrows)
        Md.apply(U.Vector(ctx, x), y)
        np.testing.assert_allclose(y.numpy(), M @ x, rtol=1e-14, atol=1e-14)


def test_stencil_operators_use_diagonal_slices(ctx):
    for A in (P.laplacian_3d(32), P.lognormal_diffusion_3d(16, 1)[0], P.laplacian_3d(96, 96, 8)):
        info = U.SparseMatrix(ctx, A).sell_info()
        assert info["ndiag_slices"] == info["nslices"]
        assert info["nstored"] == expected_diagonal_slots(A, info["rows_per_slice"])
    # 192-wide x-lines (the 192^3 workload): padding stays below 1% of the nonzeros
    A = P.laplacian_3d(192, 192, 4)
    info = U.SparseMatrix(ctx, A).sell_info()
    assert info["nstored"] <= 1.01 * A.nnz
    info = U.SparseMatrix(ctx, P.interpolation_3d(16)).sell_info()
    assert info["ndiag_slices"] < info["nslices"]


@pytest.mark.parametrize("dtype", [U.F32, U.BF16])
def test_spmv_low_precision_storage(ctx, dtype):
    A = P.lognormal_diffusion_3d(20, 3)[0]
    x = np.random.default_rng(2).standard_normal(A.ncols).astype(np.float32)
    M = U.SparseMatrix(ctx, A).cast(dtype)
    vals = A.values.astype(np.float32).astype(np.float64) if dtype == U.F32 else bf16_round(A.values)
    ref = P.CSR(A.nrows, A.ncols, A.rowptr, A.colidx, vals).matvec(x.astype(np.float64))
    vx, vy = U.Vector(ctx, x, dtype=U.F32), U.Vector(ctx, n=A.nrows, dtype=U.F32)
    M.apply(vx, vy)
    bound = 1e-6 * (np.abs(P.CSR(A.nrows, A.ncols, A.rowptr, A.colidx, vals).to_scipy()) @ np.abs(x))
    assert np.all(np.abs(vy.numpy() - ref) <= 4 * bound + 1e-30)


def test_residual_add_and_jacobi(ctx):
    A = P.lognormal_diffusion_3d(16, 4)[0]
    rng = np.random.default_rng(3)
    x, b = rng.standard_normal(A.nrows), rng.standard_normal(A.nrows)
    M = U.SparseMatrix(ctx, A)
    vx, vb, vr = U.Vector(ctx, x), U.Vector(ctx, b), U.Vector(ctx, n=A.nrows)
    Ax = A.matvec(x)
    M.residual(vb, vx, vr)
    np.testing.assert_allclose(vr.numpy(), b - Ax, rtol=1e-12, atol=1e-12 * np.abs(Ax).max())
    M.apply_add(vx, vb, vr)
    np.testing.assert_allclose(vr.numpy(), Ax + b, rtol=1e-12, atol=1e-12 * np.abs(Ax).max())
    d = A.to_scipy().diagonal()
    vo = U.Vector(ctx, n=A.nrows)
    M.jacobi_sweep(vb, vx, 0.8, vo)
    np.testing.assert_allclose(vo.numpy(), x + 0.8 / d * (b - Ax), rtol=1e-12, atol=1e-12)
    vd = U.Vector(ctx, n=A.nrows)
    M.diag(vd)
    np.testing.assert_array_equal(vd.numpy(), d)


def test_bad_csr_is_rejected(ctx):
    bad_col = P.CSR(2, 2, np.array([0, 1, 2]), np.array([0, 5]), np.array([1.0, 1.0]))
    with pytest.raises(U.UgpuError):
        U.SparseMatrix(ctx, bad_col)
    unsorted = P.CSR(1, 3, np.array([0, 2]), np.array([2, 0]), np.array([1.0, 1.0]))
    with pytest.raises(U.UgpuError):
        U.SparseMatrix(ctx, unsorted)
    bad_ptr = P.CSR(2, 2, np.array([0, 3, 2]), np.array([0, 1]), np.array([1.0, 1.0]))
    with pytest.raises(U.UgpuError):
        U.SparseMatrix(ctx, bad_ptr)


def _same_csr(gpu_mat, ora_mat, values="exact"):
    rp, ci, v = gpu_mat.csr()
    orp, oci, ov = ora_mat.arrays()
    assert (rp == orp).all() and (ci == oci).all()
    if values == "exact":
        np.testing.assert_array_equal(v, ov)
    else:
        np.testing.assert_allclose(v, ov, rtol=1e-12, atol=1e-12 * np.abs(ov).max())


@pytest.mark.parametrize("name", ["interp", "random", "random_long_rows", "empty_rows"])
def test_transpose_bit_exact(ctx, oracle, name):
    A = MATRICES[name]()
    _same_csr(U.SparseMatrix(ctx, A).transpose(), oracle.Matrix(A).transpose(), "exact")


def test_spgemm_structure_bit_exact(ctx, oracle):
    A = random_csr(800, 900, 0.01, 5)
    B = random_csr(900, 700, 0.01, 6)
    _same_csr(U.SparseMatrix(ctx, A).matmul(U.SparseMatrix(ctx, B)), oracle.Matrix(A).matmul(oracle.Matrix(B)),
              "close")


def test_spgemm_long_rows_use_the_cta_path(ctx, oracle):
    A = random_csr(300, 400, 0.02, 8, long_rows=3)
    B = random_csr(400, 500, 0.02, 9)
    _same_csr(U.SparseMatrix(ctx, A).matmul(U.SparseMatrix(ctx, B)), oracle.Matrix(A).matmul(oracle.Matrix(B)),
              "close")


def test_spgemm_wide_rows_use_the_window_path(ctx, oracle):
    """Rows with more than 4096 intermediate products (here up to ~60,000, spread over ~30,000
    columns, i.e. several 8192-column windows) go through the windowed dense-accumulator path:
    identical structure to the oracle's product and values to rounding, and identical bits on a
    second run (the accumulation order is fixed)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(21)
    A = sp.random(400, 3000, density=0.002, random_state=rng, format="lil")
    for r in (0, 7, 399):
        cols = rng.choice(3000, 2500, replace=False)
        A[r, cols] = rng.standard_normal(cols.size)
    A = A.tocsr()
    A.sort_indices()
    B = sp.random(3000, 30000, density=0.0008, random_state=rng, format="csr")
    B.sort_indices()
    Ac, Bc = P.CSR.from_scipy(A), P.CSR.from_scipy(B)
    assert (A.astype(bool).astype(int) @ np.diff(B.indptr)).max() > 4096
    Ag, Bg = U.SparseMatrix(ctx, Ac), U.SparseMatrix(ctx, Bc)
    C1 = Ag.matmul(Bg)
    _same_csr(C1, oracle.Matrix(Ac).matmul(oracle.Matrix(Bc)), "close")
    np.testing.assert_array_equal(C1.csr()[2], Ag.matmul(Bg).csr()[2])


def test_spgemm_mid_tier_and_its_overflow(ctx, oracle):
    """Rows of 129..1024 products go to the mid tier sized by distinct columns: rows whose
    products land on a few dozen columns stay there, rows with more than 128 distinct columns
    overflow to the full-size warp tier.  Both kinds in one product (666 and 667 rows): the
    oracle's structure and values, and the same bits on a second run."""
    import scipy.sparse as sp

    rng = np.random.default_rng(31)
    n, m = 2000, 3000
    rows, cols = [], []
    for i in range(n):
        k = 24 if i % 3 else 6  # 24 entries: ~24 x 20 products; 6: tier 1
        rows += [i] * k
        if i % 3 == 1:  # only B's concentrated rows: the products land on at most 40 columns
            cols += list(2 * rng.choice(m // 2, k, replace=False))
        else:
            cols += list(rng.choice(m, k, replace=False))
    A = sp.csr_matrix((rng.standard_normal(len(rows)), (rows, cols)), shape=(n, m))
    # B: half the rows concentrated on 40 columns (few distinct products), half spread (many)
    brows, bcols = [], []
    for j in range(m):
        pool = 40 if j % 2 == 0 else 2500
        c = rng.choice(pool, 20, replace=False) + (0 if j % 2 == 0 else 40)
        brows += [j] * 20
        bcols += list(c)
    B = sp.csr_matrix((rng.standard_normal(len(brows)), (brows, bcols)), shape=(m, 2540))
    A.sort_indices()
    B.sort_indices()
    C = (A @ B).tocsr()
    per_row = np.diff(C.indptr)
    ub = A.astype(bool).astype(int) @ np.diff(B.indptr)
    mid = (ub > 128) & (ub <= 1024)
    assert (mid & (per_row <= 128)).any() and (mid & (per_row > 128)).any()
    Ac, Bc = P.CSR.from_scipy(A), P.CSR.from_scipy(B)
    Ag, Bg = U.SparseMatrix(ctx, Ac), U.SparseMatrix(ctx, Bc)
    C1 = Ag.matmul(Bg)
    _same_csr(C1, oracle.Matrix(Ac).matmul(oracle.Matrix(Bc)), "close")
    np.testing.assert_array_equal(C1.csr()[2], Ag.matmul(Bg).csr()[2])


def test_ptap_structure_bit_exact_fixture(ctx, oracle, laplace_hierarchy):
    A, Is, _ = laplace_hierarchy
    _same_csr(U.SparseMatrix(ctx, A).ptap(U.SparseMatrix(ctx, Is[2])), oracle.Matrix(A).ptap(oracle.Matrix(Is[2])),
              "close")


def test_ptap_full_size_128(ctx):
    """Galerkin product at the 128^3 configuration: 64^3 coarse operator with the
    27-point structure (nnz = 190^3 = 6,859,000), symmetric, and row sums of
    P^T A P equal to P^T (A (P 1))."""
    A = P.laplacian_3d(128)
    Pm = P.interpolation_3d(128)
    Ac = U.SparseMatrix(ctx, A).ptap(U.SparseMatrix(ctx, Pm))
    assert Ac.nrows == 64 ** 3 and Ac.nnz == 190 ** 3
    rp, ci, v = Ac.csr()
    S = P.CSR(Ac.nrows, Ac.ncols, rp, ci, v).to_scipy()
    assert abs(S - S.T).max() <= 1e-12
    one = np.ones(Pm.ncols)
    ref = Pm.to_scipy().T @ (A.to_scipy() @ (Pm.to_scipy() @ one))
    np.testing.assert_allclose(S @ one, ref, rtol=1e-12, atol=1e-12)


def test_ptap_reuse_recomputes_values_in_place(ctx):
    """MatPtAP with MAT_REUSE_MATRIX (ugpu_ptap_reuse): after the values of A and P change, the
    in-place product has the bits of a fresh product; a changed structure is refused."""
    A = P.lognormal_diffusion_3d(24, 5)[0]
    Pm = P.interpolation_3d(24)
    Ag, Pg = U.SparseMatrix(ctx, A), U.SparseMatrix(ctx, Pm)
    Ac = Ag.ptap_reuse(Pg)
    ref0 = Ag.ptap(Pg).csr()
    for a, b in zip(Ac.csr(), ref0):
        np.testing.assert_array_equal(a, b)
    rng = np.random.default_rng(3)
    Ag.update_values(A.values * rng.uniform(0.5, 2.0, A.nnz))
    pv = Pm.values.copy()
    pv[rng.choice(Pm.nnz, Pm.nnz // 3, replace=False)] = 0.0  # rows truncated, structure kept
    Pg.update_values(pv)
    out = Ag.ptap_reuse(Pg, out=Ac)
    assert out is Ac
    ref = Ag.ptap(Pg).csr()
    for a, b in zip(Ac.csr(), ref):
        np.testing.assert_array_equal(a, b)
    # the reused product is a working operator (its SpMV layout was refreshed)
    x = U.Vector(ctx, rng.standard_normal(Ac.ncols))
    y, y2 = U.Vector(ctx, n=Ac.nrows), U.Vector(ctx, n=Ac.nrows)
    Ac.apply(x, y)
    U.SparseMatrix(ctx, P.CSR(Ac.nrows, Ac.ncols, *ref)).apply(x, y2)
    np.testing.assert_array_equal(y.numpy(), y2.numpy())
    with pytest.raises(U.UgpuError):  # another structure
        U.SparseMatrix(ctx, P.lognormal_diffusion_3d(24, 5)[0]).ptap_reuse(U.SparseMatrix(ctx, P.interpolation_3d(24)),
                                                                            out=U.SparseMatrix(ctx, P.laplacian_3d(12)))
    import scipy.sparse as sp

    Bs = A.to_scipy() + sp.eye(A.nrows, k=2) + sp.eye(A.nrows, k=-2)  # same size, another pattern
    with pytest.raises(U.UgpuError):  # A with another structure than the product was formed from
        U.SparseMatrix(ctx, P.CSR.from_scipy(Bs)).ptap_reuse(Pg, out=Ac)


@pytest.mark.parametrize("dtype", [U.F64, U.F32, U.BF16])
@pytest.mark.parametrize("name", ["lognormal", "interp", "random"])
def test_update_values_refreshes_the_spmv_layout(ctx, dtype, name):
    """New values through ugpu_mat_update_values reach every SpMV layout (the sliced-ELL values are
    refilled on the kept slice keys): the product equals a matrix created with those values."""
    A = MATRICES[name]()
    M = U.SparseMatrix(ctx, A)
    if dtype != U.F64:
        M = M.cast(dtype)
    v2 = A.values * np.random.default_rng(9).uniform(-2.0, 2.0, A.nnz)
    M.update_values(v2)
    ref = U.SparseMatrix(ctx, P.CSR(A.nrows, A.ncols, A.rowptr, A.colidx, v2))
    if dtype != U.F64:
        ref = ref.cast(dtype)
    vt = U.F64 if dtype == U.F64 else U.F32
    x = U.Vector(ctx, np.random.default_rng(2).standard_normal(A.ncols).astype(np.float32 if vt == U.F32 else np.float64),
                 dtype=vt)
    y1, y2 = U.Vector(ctx, n=A.nrows, dtype=vt), U.Vector(ctx, n=A.nrows, dtype=vt)
    M.apply(x, y1)
    ref.apply(x, y2)
    np.testing.assert_array_equal(y1.numpy(), y2.numpy())


def test_fp64_rate_measurement(ctx):
    """The FP64 rates the benchmark divides by: DFMA chains and the FP64 mma.sync path, both in
    the range a GB300 can deliver (about 1.2 TFLOP/s; the check only rejects nonsense)."""
    dfma, dmma = ctx.fp64_rate("dfma"), ctx.fp64_rate("dmma")
    print(f"FP64 DFMA {dfma / 1e12:.3f} TFLOP/s, DMMA m8n8k4 {dmma / 1e12:.3f} TFLOP/s")
    assert 0.2e12 < dfma < 5e12
    assert 0.2e12 < dmma < 5e12
