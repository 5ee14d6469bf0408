"""Failure detection without a GPU fault: the shared-memory staged SpMV waits for its bulk copies
with a bounded mbarrier wait.  Through a test-only entry point the product runs with a short
limit (about a millisecond) and one stage's copies are never issued, so that wait runs out: the
kernel must record the context's error flag, let its other copies land and return; the next
synchronising call must report the error (and clear it), and the context must stay usable."""
import ctypes as C

import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [U.F32, U.BF16])
def test_staged_wait_runs_out_and_the_context_stays_usable(ctx, dtype):
    A = P.lognormal_diffusion_3d(48, 2)[0]
    M = U.SparseMatrix(ctx, A).cast(dtype)
    assert M.sell_interleaved()
    xh = np.random.default_rng(3).standard_normal(A.ncols).astype(np.float32)
    x = U.Vector(ctx, xh, dtype=U.F32)
    y = U.Vector(ctx, n=A.nrows, dtype=U.F32)
    lib = ctx.lib
    launched = C.c_int(0)
    rc = lib.ugpu_test_staged_wait_timeout(M.h, x.h, y.h, 2_000_000, C.byref(launched))
    assert rc == 0, lib.ugpu_last_error(ctx.h)
    assert launched.value == 1  # the operator ran through the staged kernel
    rc = lib.ugpu_synchronize(ctx.h)
    assert rc < 0
    assert b"timed out" in lib.ugpu_last_error(ctx.h)
    assert lib.ugpu_synchronize(ctx.h) == 0  # the flag was cleared
    # the context still works: an ordinary product through the same kernel is correct
    M.apply(x, y)
    ctx.synchronize()
    vals = M.csr()[2]
    ref = P.CSR(A.nrows, A.ncols, A.rowptr, A.colidx, vals).matvec(xh.astype(np.float64))
    np.testing.assert_allclose(y.numpy(), ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())
