"""The allocation-free fused dots (ugpu_dots_noalloc) against the regular entry point.

Callers that cannot allocate device memory -- host codes whose device memory belongs to
their own pool or memory space, and hot loops that cannot afford cudaFree's device-wide
synchronisation -- use ugpu_dots_noalloc, whose scratch is a fixed array inside the
library.  This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import utopia_gb300 as U
from utopia_gb300 import _abi

pytestmark = pytest.mark.gpu


def _noalloc(lib, pairs, n, out_vec, stream):
    k = len(pairs)
    a = (C.c_void_p * k)(*[p[0].device_ptr for p in pairs])
    b = (C.c_void_p * k)(*[p[1].device_ptr for p in pairs])
    da = (C.c_int * k)(*[p[0].dtype for p in pairs])
    db = (C.c_int * k)(*[p[1].dtype for p in pairs])
    return lib.ugpu_dots_noalloc(k, a, b, da, db, n, C.c_void_p(out_vec.device_ptr), C.c_void_p(stream))


def test_dots_noalloc_matches_ugpu_dots(ctx):
    lib = _abi.load()
    rng = np.random.default_rng(11)
    n = 1_000_003
    a, b, c = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n)
    va, vb, vc = U.Vector(ctx, a), U.Vector(ctx, b), U.Vector(ctx, c)
    v32 = U.Vector(ctx, c.astype(np.float32), dtype=U.F32)
    pairs = [(va, vb), (va, va), (vb, vc), (va, v32)]
    expected = U.dots(pairs)  # the existing entry point, ugpu_dots
    out = U.Vector(ctx, n=len(pairs))  # the caller owns the output
    for call in range(2):  # two calls in a row share the library's scratch array
        out.set(np.nan)
        assert _noalloc(lib, pairs, n, out, ctx.stream) == 0, lib.ugpu_last_error(None)
        ctx.synchronize()
        got = out.numpy()
        np.testing.assert_allclose(got, expected, rtol=1e-12, atol=0)
        ref = [a @ b, a @ a, b @ c, a @ c.astype(np.float32).astype(np.float64)]
        np.testing.assert_allclose(got, ref, rtol=1e-10)


def test_dots_noalloc_allocates_nothing(ctx):
    """After a first call (which loads the library's device module in this context), a
    batch of calls leaves the device's free memory unchanged: nothing is allocated."""
    import torch

    lib = _abi.load()
    rng = np.random.default_rng(12)
    n = 300_001
    va, vb = U.Vector(ctx, rng.standard_normal(n)), U.Vector(ctx, rng.standard_normal(n))
    out = U.Vector(ctx, n=2)
    assert _noalloc(lib, [(va, vb), (vb, vb)], n, out, ctx.stream) == 0
    ctx.synchronize()
    first = out.numpy()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(50):
        assert _noalloc(lib, [(va, vb), (vb, vb)], n, out, ctx.stream) == 0
    ctx.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    np.testing.assert_array_equal(out.numpy(), first)  # deterministic call to call


def test_dots_noalloc_limits(ctx):
    lib = _abi.load()
    v = U.Vector(ctx, np.ones(10))
    out = U.Vector(ctx, n=9)
    rc = _noalloc(lib, [(v, v)] * 9, 10, out, ctx.stream)  # 9 pairs exceed the fixed scratch
    assert rc == -2 and b"scratch" in lib.ugpu_last_error(None)
    assert _noalloc(lib, [(v, v)], 0, out, ctx.stream) == 0  # empty vectors: dot = 0
    ctx.synchronize()
    assert out.numpy()[0] == 0.0
