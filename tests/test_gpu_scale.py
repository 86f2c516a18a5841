"""GPU parity at benchmark scale: the batched chain's tracklets and offsets
against the CPU oracle (pinned to the reference kernels) on the workloads
the benchmark times -- 100 pile-up-50 events in one launch, 16 and 64
pile-up-200 events, the grids the autotuner picks for pile-up 200 -- and the
serving stream's results against the oracle.  Bit-exact: integer index
sets, equality is the tolerance."""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300.ops import Pipeline

pytestmark = pytest.mark.gpu


def oracle_trk(b, w, grid=None, threads=16):
    g = grid if grid is not None else w.grid(b.n_events)
    r = oracle.run(b, w.config(), g, 4, n_threads=1, omp_threads=threads)
    assert r["stats"]["status"] == 0
    return oracle.canonical(r)["tracklets"], r["trk_offsets"], r["stats"]


def pipeline_for(ctx, w, b, grid=None, per_hit=(48, 96, 8)):
    N = b.n_hits
    g = grid if grid is not None else w.grid(b.n_events)
    return Pipeline(ctx, w.config(), g, b.n_events, N, *[k * N + 4096 for k in per_hit])


@pytest.mark.parametrize("name,n_ev", [("pileup50-batch100", 100), ("pileup200", 16)])
def test_batched_chain_equals_oracle_at_scale(gpu_ctx, name, n_ev):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    p = pipeline_for(gpu_ctx, w, b)
    trk, off, counts = p.seed(b)
    assert counts["status"] == 0
    want, want_off, st = oracle_trk(b, w)
    assert len(want) > 1000
    assert np.array_equal(trk, want)
    assert np.array_equal(off, want_off)
    assert counts["n_pairs"] == st["pairs"] and counts["pair_slots"] == st["pair_slots"]
    assert counts["n_candidates"] == st["cands"] and counts["cand_slots"] == st["cand_slots"]
    assert counts["cand_truncated"] == st["cand_truncated"]


def test_pileup200_64_events_streaming_equals_oracle(gpu_ctx):
    """The benchmark's streaming form (two batches in flight) on 64
    pile-up-200 events, 1.6 M hits, against the oracle."""
    w = gen.WORKLOADS["pileup200"]
    b = gen.generate_batch(w, 64, first_event=1000)
    p = pipeline_for(gpu_ctx, w, b)
    t1 = p.submit(b)
    t2 = p.submit(b)
    trk1, off1, c1 = p.wait(t1)
    trk2, off2, c2 = p.wait(t2)
    assert c1["status"] == 0 and np.array_equal(trk1, trk2) and np.array_equal(off1, off2)
    want, want_off, _ = oracle_trk(b, w)
    assert np.array_equal(trk1, want)
    assert np.array_equal(off1, want_off)


def test_batched_calls_do_not_read_detector_and_hit_ids(gpu_ctx):
    """The batched calls upload x, y, z, layer and event only: null detector
    and hit id columns, or columns of garbage, give the oracle's tracklets
    through trax_seed_batch and trax_submit_batch alike."""
    import dataclasses
    w = gen.WORKLOADS["pileup200"]
    b = gen.generate_batch(w, 8, first_event=77)
    want, want_off, _ = oracle_trk(b, w)
    p = pipeline_for(gpu_ctx, w, b)
    junk = np.full(b.n_hits, 0xDEADBEEF, dtype=np.uint32)
    for ids in (None, junk):
        nb = dataclasses.replace(b, detector_id=ids, hit_id=ids)
        trk, off, counts = p.seed(nb)
        assert counts["status"] == 0
        assert np.array_equal(trk, want) and np.array_equal(off, want_off)
        t1 = p.submit(nb)
        t2 = p.submit(nb)
        for t in (t1, t2):
            trk, off, counts = p.wait(t)
            assert counts["status"] == 0
            assert np.array_equal(trk, want) and np.array_equal(off, want_off)


@pytest.mark.parametrize("zp", [(64, 64), (64, 128), (32, 64), (256, 192), (320, 192), (128, 128)])
def test_autotuned_grids_equal_oracle(gpu_ctx, zp):
    """The grids the autotuner selects on pile-up 200 (the truncated
    candidate set depends on the grid, so the oracle runs at the same one),
    with every walk setting the tuner tries."""
    from trax_gb300.autotune import WALK_CANDIDATES
    w = gen.WORKLOADS["pileup200"]
    b = gen.generate_batch(w, 8, first_event=2000)
    g = gen.Workload(w.name, w.config_id, w.n_layers, w.noise, w.pt_range, zp[0], zp[1],
                     w.n_triplets, pileup_mean=w.pileup_mean)
    grid = g.grid(b.n_events)
    want, want_off, _ = oracle_trk(b, g, grid)
    p = pipeline_for(gpu_ctx, g, b, grid)
    for rw, zi in WALK_CANDIDATES[:4]:
        for rec in (3, 4, 1):
            gpu_ctx.set_tuning(rw, zi, rec)
            trk, off, counts = p.seed(b)
            assert counts["status"] == 0
            assert np.array_equal(trk, want), (rw, zi, rec)
            assert np.array_equal(off, want_off)
    gpu_ctx.set_tuning(48, 16, 3)


@pytest.mark.parametrize("zp,tuning", [(None, None), ((256, 192), (1 << 30, 256, 2))])
def test_serving_stream_equals_oracle(gpu_ctx, zp, tuning):
    """Events of the streaming workload (pile-up ~ U{0..200}) arriving as a
    Poisson stream through the continuous-batching server, at the workload's
    grid and at the tuned grid and walk the benchmark serves with: every
    event's tracklets equal the oracle's for that event alone."""
    from trax_gb300.serve import Server, poisson_arrivals
    w = gen.WORKLOADS["stream-pileup-u200"]
    if zp is not None:
        w = gen.Workload(w.name, w.config_id, w.n_layers, w.noise, w.pt_range, zp[0], zp[1],
                         w.n_triplets, pileup_uniform=w.pileup_uniform)
    events = [gen.generate_batch(w, 1, first_event=300 + i) for i in range(24)]
    # the server never reads the detector and hit ids: half the requests leave them out
    import dataclasses
    reqs = [dataclasses.replace(e, detector_id=None, hit_id=None) if i % 2 else e
            for i, e in enumerate(events)]
    cfg = w.config()
    with Server(cfg, w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=3,
                max_batch_events=8, memory_budget_bytes=6 << 30, tuning=tuning) as srv:
        t0 = srv.now_ns() + 20_000_000
        arrivals = poisson_arrivals(len(events), 2000.0, t0, seed=5)
        tickets = [srv.submit(e, int(a)) for e, a in zip(reqs, arrivals)]
        got = {}
        while len(got) < len(events):
            r = srv.poll(timeout_ms=20_000)
            assert r is not None, "server stalled"
            assert r["status"] == 0
            got[r["ticket"]] = r
    for t, e in zip(tickets, events):
        r = oracle.run(e, cfg, w.grid(1), 4, n_threads=1, omp_threads=8)
        so = r["sorted_orig"]
        want = np.stack([so[r["trk_h1"]], so[r["trk_h2"]], so[r["trk_h3"]]], axis=1) \
            if r["trk_h1"].size else np.zeros((0, 3), np.uint32)
        assert np.array_equal(got[t]["tracklets"], want)


@pytest.mark.parametrize("zp,zscale", [((64, 128), 8.0), ((64, 128), 1.0), ((48, 96), 10.0)])
def test_grid_build_in_row_bands_equals_oracle(gpu_ctx, zp, zscale):
    """Fine grids whose cell tables do not fit shared memory are built in
    bands of z rows.  Hits stretched along z (x zscale) occupy most rows and
    so several bands; the grid, the sorted order and the tracklets equal the
    oracle's."""
    w0 = gen.WORKLOADS["multimuon-1000trk"]
    w = gen.Workload(w0.name, w0.config_id, w0.n_layers, w0.noise, w0.pt_range, zp[0], zp[1],
                     w0.n_triplets, tracks=w0.tracks)
    b = gen.generate_batch(w, 3)
    b.z = (b.z * np.float32(zscale)).astype(np.float32)
    grid = w.grid(b.n_events)
    r = oracle.run(b, w.config(), grid, 4, n_threads=1, omp_threads=8)
    assert r["stats"]["status"] == 0
    p = pipeline_for(gpu_ctx, w, b, grid)
    trk, off, counts = p.seed(b)
    assert counts["status"] == 0
    assert np.array_equal(trk, oracle.canonical(r)["tracklets"])
    assert np.array_equal(off, r["trk_offsets"])
    # the stage call's grid and sorted order as well
    from trax_gb300.ops import build_triplets
    hits, g, _, _, _ = build_triplets(gpu_ctx, b, w.config(), zp[0], zp[1])
    assert np.array_equal(g.download(), r["grid"])
    assert np.array_equal(hits.download()["orig"], r["sorted_orig"])


@pytest.mark.parametrize("name,n_ev,sigma_z", [("pileup200", 16, None),
                                               ("multimuon-1000trk", 2, 4.0),
                                               ("multimuon-1000trk", 2, 30.0)])
def test_unindexed_walks_and_wide_windows_equal_oracle(gpu_ctx, name, n_ev, sigma_z):
    """Walks that never search a cell's z index (index_min 256), contiguous
    over whole runs or cell by cell.  A z window of 30 cm passes nearly every
    hit of a 50 cm row through the half-precision screen, so every screen
    step has 8 survivors and most pairs emit more candidates than a store
    record carries (the store pass walks them); the counts, the truncation
    and the tracklets equal the oracle's."""
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev, first_event=4000)
    cfg = w.config()
    if sigma_z is not None:
        for i in range(cfg.n_layer_triplets):
            cfg.triplets[i].sigma_z = sigma_z
    r = oracle.run(b, cfg, w.grid(n_ev), 4, n_threads=1, omp_threads=16)
    assert r["stats"]["status"] == 0
    want = oracle.canonical(r)["tracklets"]
    N = b.n_hits
    p = Pipeline(gpu_ctx, cfg, w.grid(n_ev), n_ev, N, 48 * N + 4096, 160 * N + 4096, 8 * N + 4096)
    try:
        for rw, rec in ((1 << 30, 2), (96, 3), (0, 1)):
            gpu_ctx.set_tuning(rw, 256, rec)
            trk, off, counts = p.seed(b)
            assert counts["status"] == 0
            assert np.array_equal(trk, want), rw
            assert np.array_equal(off, r["trk_offsets"])
            assert counts["n_candidates"] == r["stats"]["cands"]
            assert counts["cand_slots"] == r["stats"]["cand_slots"]
            assert counts["cand_truncated"] == r["stats"]["cand_truncated"]
    finally:
        gpu_ctx.set_tuning(48, 16, 3)
