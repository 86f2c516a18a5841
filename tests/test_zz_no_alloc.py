"""The allocation-free prefix sum, for callers that cannot call cudaMalloc
(code inside another framework's memory pool or allocator lock, or inside a
stream capture).  It must give the same result as the context-based
trax_prefix_sum, call after call, although its scratch is one device array
that every call clears and reuses.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(ctx, d_in, d_out, n, d_total):
    st = ctx.lib.trax_prefix_sum_noalloc(d_in.ptr, d_out.ptr, n, d_total.ptr,
                                         ctx.lib.trax_ctx_get_stream(ctx.h))
    if st != 0:
        raise AssertionError(ctx.lib.trax_prefix_sum_noalloc_error().decode())
    ctx.synchronize()


def test_noalloc_matches_prefix_sum_twice(gpu_ctx):
    ctx = gpu_ctx
    rng = np.random.default_rng(11)
    for n in (1_000_003, 4096):  # two calls in a row, the second smaller
        v = rng.integers(0, 1000, n).astype(np.uint32)
        d_in = ctx.upload(v)
        ref_out, ref_tot = ctx.alloc(n), ctx.alloc(1)
        ctx.prefix_sum(d_in, ref_out, n, ref_tot)
        out, tot = ctx.alloc(n), ctx.alloc(1)
        _noalloc(ctx, d_in, out, n, tot)
        # integer scan: exact equality is the tolerance
        assert np.array_equal(out.download(n), ref_out.download(n))
        assert tot.download(1)[0] == ref_tot.download(1)[0] == int(v.astype(np.uint64).sum())


def test_noalloc_rejects_oversize(gpu_ctx):
    ctx = gpu_ctx
    big = 8388608 + 1
    st = ctx.lib.trax_prefix_sum_noalloc(C.c_void_p(16), C.c_void_p(16), big, None, None)
    assert st == 1
    assert b"TRAX_PREFIX_SUM_NOALLOC_MAX" in ctx.lib.trax_prefix_sum_noalloc_error()
