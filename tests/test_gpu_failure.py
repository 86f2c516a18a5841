"""Failure detection on the GPU without a fault: a bounded device-side wait
is made to run out, the kernel reports it through the context's status word
and returns, and the same context then runs the seeding chain correctly.

The wait is the decoupled look-back of the scan kernel: the self-test entry
point starts the tile tickets at 1, so tile 1 waits for a tile 0 that no
block ever takes, with a limit of a few thousand polls."""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300.ops import build_triplets

pytestmark = pytest.mark.gpu

TRAX_ERR_TIMEOUT = 3
TRAX_DETAIL_SCAN_TIMEOUT = 7


def test_lookback_wait_gives_up_and_context_stays_usable(gpu_ctx):
    ctx = gpu_ctx
    n = 4096 * 6 + 17
    d_in = ctx.upload(np.ones(n, np.uint32))
    d_out = ctx.alloc(n)
    ctx.reset_counts()
    st = ctx.lib.trax_selftest_lookback_timeout(ctx.h, d_in.ptr, d_out.ptr, n, 2000)
    assert st == 0
    # synchronising returns the device status word: the wait gave up
    assert ctx.lib.trax_ctx_synchronize(ctx.h) == TRAX_ERR_TIMEOUT
    c = ctx.counts()
    assert c["status"] == TRAX_ERR_TIMEOUT and c["error_detail"] == TRAX_DETAIL_SCAN_TIMEOUT, c

    # the context keeps working: a normal scan and the whole chain
    ctx.reset_counts()
    assert ctx.counts()["status"] == 0
    ctx.prefix_sum(d_in, d_out, n)
    ctx.synchronize()
    assert np.array_equal(d_out.download(n), np.arange(n, dtype=np.uint32))
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 2)
    cfg = w.config()
    _, _, _, _, trk = build_triplets(ctx, b, cfg, w.n_sectors_z, w.n_sectors_phi)
    got = trk.hits()
    ref = oracle.run(b, cfg, w.grid(2), 4, n_threads=1)
    assert np.array_equal(got, oracle.canonical(ref)["tracklets"])
    assert ctx.counts()["status"] == 0


def test_selftest_rejects_bad_arguments(gpu_ctx):
    ctx = gpu_ctx
    d = ctx.alloc(8192)
    assert ctx.lib.trax_selftest_lookback_timeout(ctx.h, d.ptr, d.ptr, 100, 10) == 1
    assert ctx.lib.trax_selftest_lookback_timeout(ctx.h, d.ptr, d.ptr, 8192, 0) == 1
