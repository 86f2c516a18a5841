"""Streaming submission (trax_submit_batch / trax_wait_batch): two batches in
flight, uploads overlapping the previous batch's chain, results written by
the device into pinned host buffers -- every batch's result equals the
synchronous trax_seed_batch result and the oracle's."""
import ctypes as C

import numpy as np
import pytest

import oracle
from trax_gb300 import _abi as A
from trax_gb300 import gen
from trax_gb300.ops import Pipeline

pytestmark = pytest.mark.gpu


def _batches():
    w = gen.WORKLOADS["multimuon-1000trk"]
    sizes = (6, 3, 6, 1, 5)
    out, first = [], 0
    for n in sizes:
        out.append(gen.generate_batch(w, n, first_event=first))
        first += n
    return w, out


def test_stream_equals_sync_and_oracle(gpu_ctx):
    w, batches = _batches()
    E = max(b.n_events for b in batches)
    N = max(b.n_hits for b in batches)
    p = Pipeline(gpu_ctx, w.config(), w.grid(E), E, N, 80 * N, 80 * N, 8 * N)
    sync = [p.seed(b) for b in batches]
    for input_indices in (False, True):
        got = []
        tickets = []
        for k, b in enumerate(batches):
            tickets.append(p.submit(b, input_indices=input_indices))
            if k >= 1:
                got.append(p.wait(tickets[k - 1]))
        got.append(p.wait(tickets[-1]))
        for b, g, s in zip(batches, got, sync):
            trk, off, counts = g
            assert counts["status"] == 0
            if not input_indices:
                assert np.array_equal(trk, s[0])
                assert np.array_equal(off, s[1])
                assert counts == s[2]
            else:
                ref = p.seed(b, input_indices=True)
                assert np.array_equal(trk, ref[0])
    # the oracle, on the sorted indices of the first and last batch
    for b, s in ((batches[0], sync[0]), (batches[-1], sync[-1])):
        ref = oracle.canonical(oracle.run(b, w.config(), w.grid(b.n_events), 4, n_threads=1))
        assert np.array_equal(s[0], ref["tracklets"])


def test_third_submit_and_unknown_ticket_are_refused(gpu_ctx):
    w, batches = _batches()
    b = batches[0]
    p = Pipeline(gpu_ctx, w.config(), w.grid(b.n_events), b.n_events, b.n_hits,
                 80 * b.n_hits, 80 * b.n_hits, 8 * b.n_hits)
    t0 = p.submit(b)
    t1 = p.submit(b)
    # a third batch while two are in flight: the library refuses it
    cols = [np.ascontiguousarray(c) for c in b.columns()]
    ln = np.ascontiguousarray(b.layer_nhits.reshape(-1), dtype=np.uint32)
    bs = A.TraxEventBatch(b.n_events, b.n_layers, b.n_hits, *[c.ctypes.data for c in cols],
                          ln.ctypes.data)
    outs, off = p._stream_out[0]
    r = A.TraxBatchResult(outs[0].ptr, outs[1].ptr, outs[2].ptr, off.ptr, p.max_tracklets, 0, 0,
                          A.TraxCounts())
    t = C.c_uint32()
    st = gpu_ctx.lib.trax_submit_batch(gpu_ctx.h, C.byref(bs), C.byref(r), C.byref(t))
    assert st == 1
    assert gpu_ctx.lib.trax_wait_batch(gpu_ctx.h, t1 + 7, C.byref(r)) == 1
    a = p.wait(t0)
    c = p.wait(t1)
    assert np.array_equal(a[0], c[0])


def test_stream_capacity_error(gpu_ctx):
    w, batches = _batches()
    b = batches[0]
    p = Pipeline(gpu_ctx, w.config(), w.grid(b.n_events), b.n_events, b.n_hits,
                 80 * b.n_hits, 80 * b.n_hits, 8 * b.n_hits)
    n = len(p.seed(b)[0])
    cols = [np.ascontiguousarray(c) for c in b.columns()]
    ln = np.ascontiguousarray(b.layer_nhits.reshape(-1), dtype=np.uint32)
    bs = A.TraxEventBatch(b.n_events, b.n_layers, b.n_hits, *[c.ctypes.data for c in cols],
                          ln.ctypes.data)
    p.wait(p.submit(b))  # makes a set of pinned result buffers
    outs, off = p._stream_out[0]
    r = A.TraxBatchResult(outs[0].ptr, outs[1].ptr, outs[2].ptr, off.ptr, n - 1, 0, 0,
                          A.TraxCounts())
    t = C.c_uint32()
    assert gpu_ctx.lib.trax_submit_batch(gpu_ctx.h, C.byref(bs), C.byref(r), C.byref(t)) == 0
    assert gpu_ctx.lib.trax_wait_batch(gpu_ctx.h, t.value, C.byref(r)) == 5
    assert r.n_tracklets == n


def test_large_seed_batch_pipelines_halves(gpu_ctx):
    """trax_seed_batch runs batches of a million hits or more as two halves
    through the streaming slots; the concatenated result is the whole
    batch's (equal to one slot's run of the whole batch and to the oracle)."""
    import os
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 340)
    assert b.n_hits >= 1 << 20
    N = b.n_hits
    p = Pipeline(gpu_ctx, w.config(), w.grid(b.n_events), b.n_events, N, 80 * N, 80 * N, 8 * N)
    for input_indices in (False, True):
        trk, off, counts = p.seed(b, input_indices=input_indices)
        assert counts["status"] == 0
        whole = p.wait(p.submit(b, input_indices=input_indices))
        assert np.array_equal(trk, whole[0])
        assert np.array_equal(off, whole[1])
        assert counts == whole[2]
        if not input_indices:
            ref = oracle.canonical(oracle.run(b, w.config(), w.grid(b.n_events), 4, n_threads=1,
                                              omp_threads=os.cpu_count() or 1))
            assert np.array_equal(trk, ref["tracklets"])
