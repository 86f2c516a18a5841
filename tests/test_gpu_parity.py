"""GPU parity: the sm_103a path through the C-ABI against the CPU oracle.

Bar: bit-exact.  Grid, sorted hit columns (float bits), pairs, candidates
(as hit triples), tracklets and all per-(event, layer triplet) offsets must
equal the oracle's, element for element; the reference's slot counts
(pairCount / predictCount totals) must match too.
"""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300.ops import build_triplets, Pipeline

pytestmark = pytest.mark.gpu

CASES = [("single-muon-100trk", 1), ("single-muon-100trk", 5), ("multimuon-1000trk", 1),
         ("multimuon-1000trk", 3), ("pileup50-batch100", 3)]


def gpu_stages(ctx, b, w):
    hits, grid, pairs, cands, trk = build_triplets(ctx, b, w.config(), w.n_sectors_z,
                                                   w.n_sectors_phi)
    out = {"grid": grid.download(), "sorted": hits.download(), "pairs": pairs.get_pairings(),
           "pair_offsets": pairs.get_pairing_offsets(), "cands": cands.get_pairings(),
           "cand_offsets": cands.get_pairing_offsets(), "trk": trk.hits(),
           "trk_offsets": trk.get_tracklet_offsets(), "pair_counts": pairs_counts(pairs),
           "counts": None}
    return out


def pairs_counts(p):
    return p.count


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def cand_hits(pairs, cands):
    if cands.size == 0:
        return np.zeros((0, 3), np.uint32)
    return np.stack([pairs[cands[:, 0], 0], pairs[cands[:, 0], 1], cands[:, 1]], axis=1)


@pytest.mark.parametrize("name,n_ev", CASES)
def test_stage_parity_bit_exact(gpu_ctx, name, n_ev):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    cfg, g = w.config(), w.grid(n_ev)
    r = oracle.run(b, cfg, g, 4, n_threads=1)
    assert r["stats"]["status"] == 0
    oc = oracle.canonical(r)
    d = gpu_stages(gpu_ctx, b, w)

    assert np.array_equal(d["grid"], r["grid"])
    srt = d["sorted"]
    for col, key in (("x", "sorted_x"), ("y", "sorted_y"), ("z", "sorted_z"),
                     ("phi", "sorted_phi")):
        assert np.array_equal(bits(srt[col]), bits(r[key])), col
    for col, key in (("layer", "sorted_layer"), ("detector_id", "sorted_det"),
                     ("hit_id", "sorted_hitid"), ("event", "sorted_event"),
                     ("orig", "sorted_orig")):
        assert np.array_equal(srt[col], r[key]), col

    assert np.array_equal(d["pairs"], oc["pairs"])
    st = r["stats"]
    assert st["pairs"] == st["pair_slots"]
    assert np.array_equal(d["pair_offsets"], r["pair_offsets"])

    assert np.array_equal(cand_hits(d["pairs"], d["cands"]), oc["cand_hits"])
    if st["cands"] == st["cand_slots"]:
        assert np.array_equal(d["cand_offsets"], r["cand_offsets"])

    assert np.array_equal(d["trk"], oc["tracklets"])
    assert np.array_equal(d["trk_offsets"], r["trk_offsets"])
    assert len(d["trk"]) > 0


@pytest.mark.parametrize("name,n_ev", [("multimuon-1000trk", 2), ("pileup50-batch100", 2)])
def test_sets_equal_reference_thread_layout(gpu_ctx, name, n_ev):
    """Against the reference's default work-group size (256 threads, strided
    pair slots) the GPU's pair, candidate and tracklet sets are equal."""
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    r = oracle.run(b, w.config(), w.grid(n_ev), 4, n_threads=256)
    oc = oracle.canonical(r)
    d = gpu_stages(gpu_ctx, b, w)
    as_set = lambda a: set(map(tuple, np.asarray(a).tolist()))
    assert as_set(d["pairs"]) == as_set(oc["pairs"])
    assert as_set(cand_hits(d["pairs"], d["cands"])) == as_set(oc["cand_hits"])
    assert as_set(d["trk"]) == as_set(oc["tracklets"])
    assert np.array_equal(d["trk_offsets"], r["trk_offsets"])


def test_device_math_bit_exact(gpu_ctx):
    """The device evaluates trax_math.h to the same bits as the host."""
    import ctypes as C
    rng = np.random.default_rng(5)
    n = 1 << 20
    a = np.concatenate([rng.normal(0, 10, n - 12).astype(np.float32),
                        np.array([0, -0.0, 1, -1, np.inf, -np.inf, np.nan, 1e-40, -1e-40,
                                  3e38, -3e38, 0.5], np.float32)])
    bb = rng.normal(0, 10, n).astype(np.float32)
    u = rng.uniform(-1.05, 1.05, n).astype(np.float32)
    da, db, du = gpu_ctx.upload(a), gpu_ctx.upload(bb), gpu_ctx.upload(u)
    out = gpu_ctx.alloc(n, np.float32)
    with np.errstate(over="ignore"):
        scaled = (a * np.float32(1e9)).astype(np.float32)
    big = np.concatenate([a, scaled,
                          np.array([2.0**31, -2.0**31, 2.0**32, -3e9, 4.5e9, 2.0**40, 9.2233715e18,
                                    -9.2233715e18, 9.3e18, 2.0**62, -(2.0**62)], np.float32)])[:n]
    dbig = gpu_ctx.upload(big)
    for fn, x, y in ((0, da, db), (1, du, du), (2, da, da), (3, dbig, dbig), (4, dbig, dbig)):
        gpu_ctx._check(gpu_ctx.lib.trax_eval_math(gpu_ctx.h, fn, x.ptr, y.ptr, out.ptr, n))
        got = out.download(n)
        host = oracle.math_batch(fn, big if fn >= 3 else a if fn != 1 else u,
                                 bb if fn == 0 else None)
        # NaN results may differ in payload bits (the GPU returns the
        # canonical NaN); every other result must match bit for bit
        same = (bits(got) == bits(host)) | (np.isnan(got) & np.isnan(host))
        bad = np.nonzero(~same)[0]
        assert bad.size == 0, (fn, bad[:8], got[bad[:8]], host[bad[:8]])


def test_batched_pipeline_equals_stages(gpu_ctx):
    w = gen.WORKLOADS["pileup50-batch100"]
    b = gen.generate_batch(w, 4)
    d = gpu_stages(gpu_ctx, b, w)
    p = Pipeline(gpu_ctx, w.config(), w.grid(8), max_events=8, max_hits=b.n_hits * 2,
                 max_pairs=4 * len(d["pairs"]) + 1024, max_candidates=4 * len(d["cands"]) + 1024,
                 max_tracklets=4 * len(d["trk"]) + 1024)
    for _ in range(2):  # second call replays the captured graph
        trk, off, counts = p.seed(b)
        assert counts["status"] == 0
        assert np.array_equal(trk, d["trk"])
        assert np.array_equal(off, d["trk_offsets"])
    trk_in, _, _ = p.seed(b, input_indices=True)
    assert np.array_equal(trk_in, d["sorted"]["orig"][d["trk"]])


def test_event_alone_equals_event_in_batch(gpu_ctx):
    """Serving determinism: an event's tracklets (as input hit positions
    within the event) are the same alone and inside a batch."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 4)
    T = w.n_triplets
    p = Pipeline(gpu_ctx, w.config(), w.grid(4), max_events=4, max_hits=b.n_hits,
                 max_pairs=200_000, max_candidates=200_000, max_tracklets=50_000)
    trk, off, _ = p.seed(b, input_indices=True)
    eoff = b.event_offset
    for e in range(4):
        one = b.slice_events(e, 1)
        t1, off1, _ = p.seed(one, input_indices=True)
        lo, hi = off[e * T], off[(e + 1) * T]
        assert np.array_equal(trk[lo:hi] - eoff[e], t1)
        assert np.array_equal(off[e * T:(e + 1) * T + 1] - off[e * T], off1)


def test_empty_batch(gpu_ctx):
    w = gen.WORKLOADS["single-muon-100trk"]
    b = gen.generate_batch(w, 2)
    empty = gen.EventBatch(b.x[:0], b.y[:0], b.z[:0], b.layer[:0], b.detector_id[:0],
                           b.hit_id[:0], b.event[:0], np.zeros((2, 3), np.uint32))
    d = gpu_stages(gpu_ctx, empty, w)
    assert len(d["trk"]) == 0 and len(d["pairs"]) == 0
    assert d["trk_offsets"].tolist() == [0, 0, 0]


def test_capacity_overflow_is_reported_not_written(gpu_ctx):
    from trax_gb300.ops import PairGeneratorBeamspot, HitCollection, Grid, GridBuilder, supplements
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 1)
    cfg = w.config()
    gpu_ctx.configure(cfg)
    hits = HitCollection(gpu_ctx, b)
    es, ls = supplements(b)
    grid = Grid(gpu_ctx, 1, w.n_layers, w.n_sectors_z, w.n_sectors_phi)
    GridBuilder(gpu_ctx).run(hits, 256, es, ls, grid)
    op = PairGeneratorBeamspot(gpu_ctx)
    pairs = op.run(hits, cfg, 256, cfg, grid, capacity=100)  # grows after overflow
    r = oracle.run(b, cfg, w.grid(1), 2, n_threads=1)
    assert pairs.capacity >= pairs.count == r["stats"]["pairs"]
    assert np.array_equal(pairs.get_pairings(), oracle.canonical(r)["pairs"])


def test_bad_hit_flagged_without_fault(gpu_ctx):
    w = gen.WORKLOADS["single-muon-100trk"]
    b = gen.generate_batch(w, 1)
    b.z[5] = np.float32(400.0)  # outside the -300..300 cm grid
    d_ctx = gpu_ctx
    from trax_gb300.ops import HitCollection, Grid, GridBuilder, supplements
    d_ctx.configure(w.config())
    d_ctx.reset_counts()
    hits = HitCollection(d_ctx, b)
    es, ls = supplements(b)
    grid = Grid(d_ctx, 1, w.n_layers, w.n_sectors_z, w.n_sectors_phi)
    GridBuilder(d_ctx).run(hits, 256, es, ls, grid)
    c = d_ctx.counts()
    assert c["status"] == 6 and c["error_detail"] == 1
    d_ctx.reset_counts()
    assert d_ctx.counts()["status"] == 0


def test_tuning_does_not_change_results(gpu_ctx):
    """Walking vs index search of the candidates is a speed knob only: dense
    pile-up events give bit-identical pipelines under every setting, equal to
    the oracle."""
    w = gen.WORKLOADS["pileup50-batch100"]
    b = gen.generate_batch(w, 3)
    ref = oracle.canonical(oracle.run(b, w.config(), w.grid(3), 4, n_threads=1))["tracklets"]
    p = Pipeline(gpu_ctx, w.config(), w.grid(3), 3, b.n_hits, 60 * b.n_hits, 60 * b.n_hits,
                 8 * b.n_hits)
    outs = []
    try:
        for walk, imin, rec in ((0, 0, 1), (0, 16, 0), (48, 16, 1), (96, 32, 0),
                                (1 << 30, 256, 1), (1 << 30, 256, 0), (0, 16, 2),
                                (1 << 30, 256, 2), (0, 16, 3), (1 << 30, 256, 3),
                                (1 << 30, 256, 4), (0, 16, 4)):
            gpu_ctx.set_tuning(walk, imin, rec)
            trk, off, counts = p.seed(b)
            assert counts["status"] == 0
            outs.append(trk)
    finally:
        gpu_ctx.set_tuning(48, 16)
    for t in outs:
        assert np.array_equal(t, ref)


def test_device_reciprocal_floor_div(gpu_ctx):
    """The kernels' sector floors through 1/d equal floorf(x / d) on the
    device, next to every cell boundary of every grid size."""
    from test_oracle import floor_div_cases
    x, d = floor_div_cases()
    n = x.size
    dx, dd = gpu_ctx.upload(x), gpu_ctx.upload(d)
    out = gpu_ctx.alloc(n, np.float32)
    gpu_ctx._check(gpu_ctx.lib.trax_eval_math(gpu_ctx.h, 5, dx.ptr, dd.ptr, out.ptr, n))
    got = out.download(n)
    with np.errstate(all="ignore"):
        want = np.floor(x / d).astype(np.float32)
    same = (bits(got) == bits(want)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), x[~same][:8]


def test_full_size_batch_events_independent(gpu_ctx):
    """At the benchmark's full size (2048 multimuon events, 6.6 M hits) every
    event's tracklets equal the event run alone -- events are independent, a
    property that holds at any size -- checked on a spread of events, with
    the batch's offsets monotone and ending at the tracklet count."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    E = 2048
    b = gen.generate_batch(w, E)
    N = b.n_hits
    T = w.n_triplets
    p = Pipeline(gpu_ctx, w.config(), w.grid(E), E, N, 80 * N, 80 * N, 8 * N)
    trk, off, counts = p.seed(b, input_indices=True)
    assert counts["status"] == 0
    assert off[0] == 0 and off[-1] == len(trk) == counts["n_tracklets"]
    assert (np.diff(off.astype(np.int64)) >= 0).all()
    eoff = b.event_offset
    for e in (0, 1, 511, 1024, 1777, 2047):
        one = b.slice_events(e, 1)
        q = Pipeline(gpu_ctx, w.config(), w.grid(1), 1, one.n_hits, 80 * one.n_hits,
                     80 * one.n_hits, 8 * one.n_hits)
        t1, off1, _ = q.seed(one, input_indices=True)
        lo, hi = off[e * T], off[(e + 1) * T]
        assert np.array_equal(trk[lo:hi] - eoff[e], t1)
        assert np.array_equal(off[e * T:(e + 1) * T + 1] - off[e * T], off1)


def _drop_buckets(b, drop):
    """The batch without the hits of the (event, layer) buckets in `drop`
    (layers 1-based); the emptied buckets stay in the layout with no hits."""
    keep = np.ones(b.n_hits, bool)
    ln = b.layer_nhits.copy()
    for e, l in drop:
        keep &= ~((b.event == e) & (b.layer == l))
        ln[e, l - 1] = 0
    return gen.EventBatch(b.x[keep], b.y[keep], b.z[keep], b.layer[keep], b.detector_id[keep],
                          b.hit_id[keep], b.event[keep], ln)


def test_ragged_batch_equals_oracle(gpu_ctx):
    """Ragged batches through the batched chain: an empty first and last
    event, an empty event in the middle, and events with an empty inner,
    middle or outer layer -- tracklets and every per-(event, layer triplet)
    offset equal the oracle's."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    E, L = 7, w.n_layers
    b = gen.generate_batch(w, E)
    drop = [(0, l) for l in range(1, L + 1)] + [(3, l) for l in range(1, L + 1)] + \
           [(E - 1, l) for l in range(1, L + 1)] + [(1, 1), (2, 2), (4, 3), (5, L)]
    rb = _drop_buckets(b, drop)
    assert rb.event_nhits[0] == rb.event_nhits[3] == rb.event_nhits[E - 1] == 0
    N = rb.n_hits
    p = Pipeline(gpu_ctx, w.config(), w.grid(E), E, N, 80 * N, 80 * N, 8 * N)
    trk, off, counts = p.seed(rb)
    assert counts["status"] == 0
    r = oracle.run(rb, w.config(), w.grid(E), 4, n_threads=1)
    assert np.array_equal(trk, oracle.canonical(r)["tracklets"])
    assert np.array_equal(off, r["trk_offsets"])
    T = w.n_triplets
    for e in (0, 3, E - 1):
        assert off[e * T] == off[(e + 1) * T]
    # the same batch through the streaming slots and the per-stage calls
    st = p.wait(p.submit(rb))
    assert np.array_equal(st[0], trk) and np.array_equal(st[1], off)
    d = gpu_stages(gpu_ctx, rb, w)
    assert np.array_equal(d["trk"], trk) and np.array_equal(d["trk_offsets"], off)


def test_mixed_segment_sizes_equal_oracle(gpu_ctx):
    """One pile-up-200 event batched with multimuon events (one
    configuration): the grid build's plan follows the average segment, so
    the pile-up segments take the unstaged path that scatters each column
    while the multimuon segments are staged in shared memory -- both kinds
    in one launch, with tracklets and offsets equal to the oracle's."""
    wp = gen.WORKLOADS["pileup200"]
    wm = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.EventBatch.concat([gen.generate_batch(wp, 1), gen.generate_batch(wm, 3)])
    E, N = b.n_events, b.n_hits
    assert b.layer_nhits.max() > 2 * N / (E * b.n_layers)
    cfg = wp.config()
    p = Pipeline(gpu_ctx, cfg, wp.grid(E), E, N, 80 * N, 80 * N, 8 * N)
    trk, off, counts = p.seed(b)
    assert counts["status"] == 0
    r = oracle.run(b, cfg, wp.grid(E), 4, n_threads=1, omp_threads=4)
    assert np.array_equal(trk, oracle.canonical(r)["tracklets"])
    assert np.array_equal(off, r["trk_offsets"])
