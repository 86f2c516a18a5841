"""Continuous batching: events arriving as a Poisson stream are batched
while other batches run, and every event's result equals the event run
alone (config 5's determinism requirement)."""
import numpy as np
import pytest

from trax_gb300 import gen
from trax_gb300.ops import Pipeline
from trax_gb300.serve import Server, poisson_arrivals

pytestmark = pytest.mark.gpu


def small_stream_workload():
    w = gen.WORKLOADS["stream-pileup-u200"]
    return gen.Workload("stream-pileup-u20", 5, w.n_layers, w.noise, w.pt_range,
                        w.n_sectors_z, w.n_sectors_phi, w.n_triplets, pileup_uniform=20)


def test_results_equal_alone_and_in_mix(gpu_ctx):
    w = small_stream_workload()
    events = [gen.generate_batch(w, 1, first_event=i) for i in range(48)]
    cfg = w.config()
    # each event alone through the batched pipeline, as input positions
    p = Pipeline(gpu_ctx, cfg, w.grid(1), 1, max(e.n_hits for e in events) + 1,
                 2_000_000, 2_000_000, 400_000)
    alone = [p.seed(e, input_indices=True)[0] for e in events]
    with Server(cfg, w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=2,
                max_batch_events=16, memory_budget_bytes=2 << 30) as srv:
        t0 = srv.now_ns() + 20_000_000
        arrivals = poisson_arrivals(len(events), 5000.0, t0, seed=3)
        tickets = [srv.submit(e, int(a)) for e, a in zip(events, arrivals)]
        got = {}
        while len(got) < len(events):
            r = srv.poll(timeout_ms=10_000)
            assert r is not None, "server stalled"
            assert r["status"] == 0
            got[r["ticket"]] = r
        stats = srv.stats()
    for t, ref in zip(tickets, alone):
        assert np.array_equal(got[t]["tracklets"], ref)
    assert stats["events"] == len(events) and stats["errors"] == 0
    assert stats["batches"] < len(events)  # requests were batched together
    assert max(r["batch_events"] for r in got.values()) > 1
    assert stats["p99_ns"] >= stats["p50_ns"] > 0


def test_pair_bound_defers_instead_of_splitting(gpu_ctx):
    """A small pair capacity (one pair per hit of the batch): the counted pair
    totals keep every admitted batch within it -- requests that do not fit
    go back to the queue and lead the next batch -- so no batch overflows
    and splits, and results stay identical."""
    w = small_stream_workload()
    events = [gen.generate_batch(w, 1, first_event=100 + i) for i in range(12)]
    cfg = w.config()
    p = Pipeline(gpu_ctx, cfg, w.grid(1), 1, max(e.n_hits for e in events) + 1,
                 2_000_000, 2_000_000, 400_000)
    alone = [p.seed(e, input_indices=True)[0] for e in events]
    total = sum(e.n_hits for e in events)
    with Server(cfg, w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=1,
                max_batch_events=12, max_event_hits=total, max_batch_hits=total,
                pairs_per_hit=1, memory_budget_bytes=1 << 30) as srv:
        t0 = srv.now_ns()
        tickets = [srv.submit(e, t0) for e in events]  # all arrive at once
        got = {}
        while len(got) < len(events):
            r = srv.poll(timeout_ms=10_000)
            assert r is not None and r["status"] == 0
            got[r["ticket"]] = r
        stats = srv.stats()
    for t, ref in zip(tickets, alone):
        assert np.array_equal(got[t]["tracklets"], ref)
    assert stats["errors"] == 0
    assert stats["splits"] == 0
    assert stats["deferred"] > 0 and stats["count_passes"] >= 1
    assert stats["batches"] > 1


def test_candidate_overflow_still_splits(gpu_ctx):
    """The candidate capacity is only checked on the device: a batch whose
    candidates overflow splits in halves and reruns, results unchanged.
    Pile-up up to 60 makes about 3 candidates per hit, against a capacity
    of one per hit of the 12 events (which the densest event alone fits)."""
    w0 = gen.WORKLOADS["stream-pileup-u200"]
    w = gen.Workload("stream-pileup-u60", 5, w0.n_layers, w0.noise, w0.pt_range,
                     w0.n_sectors_z, w0.n_sectors_phi, w0.n_triplets, pileup_uniform=60)
    events = [gen.generate_batch(w, 1, first_event=200 + i) for i in range(12)]
    cfg = w.config()
    p = Pipeline(gpu_ctx, cfg, w.grid(1), 1, max(e.n_hits for e in events) + 1,
                 2_000_000, 2_000_000, 400_000)
    alone = [p.seed(e, input_indices=True)[0] for e in events]
    total = sum(e.n_hits for e in events)
    with Server(cfg, w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=1,
                max_batch_events=12, max_event_hits=total, max_batch_hits=total,
                candidates_per_hit=1, memory_budget_bytes=1 << 30) as srv:
        t0 = srv.now_ns()
        tickets = [srv.submit(e, t0) for e in events]
        got = {}
        while len(got) < len(events):
            r = srv.poll(timeout_ms=10_000)
            assert r is not None and r["status"] == 0
            got[r["ticket"]] = r
        stats = srv.stats()
    for t, ref in zip(tickets, alone):
        assert np.array_equal(got[t]["tracklets"], ref)
    assert stats["errors"] == 0
    assert stats["splits"] > 0


def test_count_pairs_batch_equals_oracle(gpu_ctx):
    """The admission count: per event the pairs the chain stores, equal to
    the oracle's distinct pairs of that event, in a batch of ragged events."""
    import ctypes as C
    import oracle
    from trax_gb300._abi import TraxEventBatch
    w = gen.WORKLOADS["stream-pileup-u200"]
    b = gen.EventBatch.concat([gen.generate_batch(w, 1, first_event=50 + i) for i in range(6)])
    N = b.n_hits
    keep = Pipeline(gpu_ctx, w.config(), w.grid(b.n_events), b.n_events, N, 48 * N, 96 * N, 8 * N)
    cols = [np.ascontiguousarray(c) for c in b.columns()]
    ln = np.ascontiguousarray(b.layer_nhits.reshape(-1), dtype=np.uint32)
    bs = TraxEventBatch(b.n_events, b.n_layers, N, *[c.ctypes.data for c in cols], ln.ctypes.data)
    out = np.zeros(b.n_events, np.uint32)
    gpu_ctx._check(gpu_ctx.lib.trax_count_pairs_batch(gpu_ctx.h, C.byref(bs), out.ctypes.data))
    for e in range(b.n_events):
        one = b.slice_events(e, 1)
        r = oracle.run(one, w.config(), w.grid(1), 2, n_threads=1, omp_threads=8)
        assert int(out[e]) == r["stats"]["pairs"]
    del keep
