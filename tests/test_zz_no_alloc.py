"""The allocation-free prefix sum (trax_prefix_sum_noalloc), called through
the C-ABI.  It serves callers that cannot call cudaMalloc where they need
the scan -- code inside another framework's memory pool or allocator
callback, code whose device memory a pool has reserved in full, paths that
cannot take cudaMalloc's implicit device synchronisation -- so its scratch
is one device array that every call clears and reuses.  It must give the
same result as the context-based trax_prefix_sum, call after call, at the
edges of its size range and in place.  The file is collected last on
purpose, and passes alone in a fresh process as well as after the rest."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 8388608  # TRAX_PREFIX_SUM_NOALLOC_MAX


def _noalloc(ctx, d_in, d_out, n, d_total):
    stream = ctx.lib.trax_ctx_get_stream(ctx.h)
    st = ctx.lib.trax_prefix_sum_noalloc(d_in.ptr if d_in else None,
                                         d_out.ptr if d_out else None, n,
                                         d_total.ptr if d_total else None, stream)
    if st != 0:
        raise AssertionError(ctx.lib.trax_prefix_sum_noalloc_error().decode())
    # the bounded look-back waits did not give up in this call
    st = ctx.lib.trax_prefix_sum_noalloc_status(stream)
    assert st == 0, ctx.lib.trax_prefix_sum_noalloc_error().decode()
    ctx.synchronize()


def _reference(ctx, d_in, n):
    out, tot = ctx.alloc(max(n, 1)), ctx.alloc(1)
    ctx.prefix_sum(d_in, out, n, tot)
    ctx.synchronize()
    return out.download(n), int(tot.download(1)[0])


def test_noalloc_matches_prefix_sum_twice(gpu_ctx):
    ctx = gpu_ctx
    rng = np.random.default_rng(11)
    for n in (1_000_003, 4096):  # two calls in a row, the second smaller
        v = rng.integers(0, 1000, n).astype(np.uint32)
        d_in = ctx.upload(v)
        want, want_tot = _reference(ctx, d_in, n)
        out, tot = ctx.alloc(n), ctx.alloc(1)
        _noalloc(ctx, d_in, out, n, tot)
        # integer scan: exact equality is the tolerance
        assert np.array_equal(out.download(n), want)
        assert int(tot.download(1)[0]) == want_tot == int(v.astype(np.uint64).sum())


def test_noalloc_at_the_maximum_size_then_in_place(gpu_ctx):
    """n == TRAX_PREFIX_SUM_NOALLOC_MAX uses every tile word of the array;
    values below 512 keep the total inside uint32.  Then an in-place scan."""
    ctx = gpu_ctx
    rng = np.random.default_rng(12)
    v = rng.integers(0, 512, NOALLOC_MAX).astype(np.uint32)
    d_in = ctx.upload(v)
    want, want_tot = _reference(ctx, d_in, NOALLOC_MAX)
    out, tot = ctx.alloc(NOALLOC_MAX), ctx.alloc(1)
    _noalloc(ctx, d_in, out, NOALLOC_MAX, tot)
    assert np.array_equal(out.download(NOALLOC_MAX), want)
    assert int(tot.download(1)[0]) == want_tot
    w = rng.integers(0, 1 << 16, 70_001).astype(np.uint32)
    d = ctx.upload(w)
    want2, want2_tot = _reference(ctx, d, w.size)
    _noalloc(ctx, d, d, w.size, tot)
    assert np.array_equal(d.download(w.size), want2)
    assert int(tot.download(1)[0]) == want2_tot


def test_noalloc_empty_input(gpu_ctx):
    ctx = gpu_ctx
    tot = ctx.upload(np.array([12345], np.uint32))
    _noalloc(ctx, None, None, 0, tot)
    assert int(tot.download(1)[0]) == 0


def test_noalloc_rejects_bad_arguments(gpu_ctx):
    ctx = gpu_ctx
    st = ctx.lib.trax_prefix_sum_noalloc(C.c_void_p(16), C.c_void_p(16), NOALLOC_MAX + 1,
                                         None, None)
    assert st == 1
    assert b"TRAX_PREFIX_SUM_NOALLOC_MAX" in ctx.lib.trax_prefix_sum_noalloc_error()
    st = ctx.lib.trax_prefix_sum_noalloc(None, None, 10, None, None)
    assert st == 1
    assert b"null" in ctx.lib.trax_prefix_sum_noalloc_error()
