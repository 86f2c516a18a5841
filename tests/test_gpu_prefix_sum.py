"""GPU PrefixSum::run counterpart against the reference's own self-check
(src/trax_test/trax_test.cpp:473-479: all ones -> out[N-1] == N-1) and the
oracle's restatement of the recursive work-group scan."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_all_ones_1mi(gpu_ctx):
    n = 1024 * 1024
    d = gpu_ctx.upload(np.ones(n, np.uint32))
    tot = gpu_ctx.alloc(1)
    gpu_ctx.prefix_sum(d, d, n, tot)  # in place, as the reference
    out = d.download(n)
    assert out[n - 1] == n - 1
    assert np.array_equal(out, np.arange(n, dtype=np.uint32))
    assert tot.download(1)[0] == n


@pytest.mark.parametrize("n", [0, 1, 2, 2047, 2048, 2049, 100_003, 3 * 2048 * 64 + 5])
def test_matches_oracle_scan(gpu_ctx, n):
    v = np.random.default_rng(n).integers(0, 1000, max(n, 1)).astype(np.uint32)[:n]
    d_in = gpu_ctx.upload(v if n else np.zeros(1, np.uint32))
    d_out = gpu_ctx.alloc(max(n, 1))
    tot = gpu_ctx.alloc(1).zero()
    gpu_ctx.prefix_sum(d_in, d_out, n, tot)
    assert gpu_ctx.counts()["status"] == 0
    want = oracle.prefix_sum(v, 256) if n else v
    assert np.array_equal(d_out.download(n), want)
    assert tot.download(1)[0] == int(v.astype(np.uint64).sum())
