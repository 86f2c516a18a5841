"""GPU event ingest (trax_ingest: HitCollection::addEvent for a batch) against
the oracle's restatement, and the whole path from event-file bytes to
tracklets."""
import numpy as np
import pytest

import oracle
from pb_util import container, events_from_batch, synth_events
from test_ingest import HAND, HAND_EXPECTED
from trax_gb300 import gen, ingest
from trax_gb300._abi import make_config
from trax_gb300.ops import build_triplets

pytestmark = pytest.mark.gpu

DET_IDS = np.arange(1000, 1400, 3, dtype=np.uint32)


def resolve(ids, det):
    """DetectorGeometry::resolveDetId (DetectorGeometry.cpp:4-30)."""
    lo, hi = 0, len(ids)
    while lo < hi:
        mid = lo + (hi - lo) // 2
        if ids[mid] < det:
            lo = mid + 1
        else:
            hi = mid
    return lo if lo < len(ids) and ids[lo] == det else -1


def oracle_batch(d, cfg, det_ids, only_tracks=True, num_tracks=-1):
    ml, mask = ingest.used_layers(cfg)
    idx, ln, trk, toff = oracle.add_events(d.layer, d.sim_track_id, d.sim_track_pt,
                                           d.hit_offset, cfg.min_pt, ml, mask, only_tracks,
                                           num_tracks)
    ev = np.repeat(np.arange(d.n_events, dtype=np.uint32), ln.sum(axis=1).astype(np.int64))
    det = np.array([r if r >= 0 else v for v, r in
                    ((int(v), resolve(det_ids, int(v))) for v in d.detector_id[idx])], np.uint32)
    b = gen.EventBatch(d.x[idx], d.y[idx], d.z[idx], d.layer[idx], det,
                       d.sim_track_id[idx], ev, ln)
    return b, trk, toff


def hand_config():
    return make_config([(1, 2, 3, 0.01, 0.037, 0.075, 0.032, 0.5, 2, 10.0, 2, 4)],
                       [4.0, 7.0, 10.0], [4.5, 7.5, 10.5], 1.0)


@pytest.mark.parametrize("key", list(HAND_EXPECTED))
def test_gpu_ingest_hand_built(gpu_ctx, key):
    only, num = key
    hits = [(float(i), 1.0, 2.0, 0, l, 5000 + i, i, t if t else None, p if t else None)
            for i, (t, l, p) in enumerate(HAND)]
    d = ingest.decode(container([(1, 1, 1, hits)]))
    b, trk = ingest.ingest(gpu_ctx, d, hand_config(), None, num_tracks=num, only_tracks=bool(only))
    want_idx, want_ln, want_trk = HAND_EXPECTED[key]
    assert b.x.tolist() == [float(i) for i in want_idx]
    assert b.layer_nhits.reshape(-1).tolist() == want_ln
    got = list(zip(trk.track_id.tolist(), trk.inner.tolist(), trk.middle.tolist(),
                   trk.outer.tolist()))
    assert got == want_trk
    assert b.detector_id.tolist() == [5000 + i for i in want_idx]


@pytest.mark.parametrize("seed,n_ev,n_trk,only,num", [
    (11, 1, 60, True, -1), (12, 7, 80, True, -1), (13, 5, 80, False, -1),
    (14, 4, 80, True, 25), (15, 3, 80, False, 10), (16, 300, 20, True, -1),
    (17, 2, 2500, True, -1), (18, 2, 2500, False, -1)])
def test_gpu_ingest_matches_oracle(gpu_ctx, seed, n_ev, n_trk, only, num):
    cfg = gen.WORKLOADS["multimuon-1000trk"].config()
    d = ingest.decode(container(synth_events(seed, n_ev, n_tracks=n_trk, det_ids=DET_IDS)))
    want, wtrk, wtoff = oracle_batch(d, cfg, DET_IDS, only, num)
    b, trk = ingest.ingest(gpu_ctx, d, cfg, DET_IDS, num_tracks=num, only_tracks=only)
    for k in ("x", "y", "z", "layer", "detector_id", "hit_id", "event"):
        assert np.array_equal(getattr(b, k), getattr(want, k)), k
    assert np.array_equal(b.layer_nhits, want.layer_nhits)
    assert np.array_equal(trk.offsets, wtoff)
    got = np.stack([trk.track_id, trk.inner, trk.middle, trk.outer], axis=1)
    assert np.array_equal(got, wtrk)
    assert len(b.x) > 0


def test_file_to_tracklets(gpu_ctx):
    """Event-file bytes -> decode -> GPU addEvent -> GPU seeding equals the
    oracle's decode -> addEvent -> seeding."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    src = gen.generate_batch(w, 3)
    pt = lambda t: 0.5 if t % 7 == 0 else 5.0  # every 7th track below min_pt
    d = ingest.decode(container(events_from_batch(src, pt)))
    cfg = w.config()
    want, _, _ = oracle_batch(d, cfg, np.zeros(0, np.uint32))
    b, _ = ingest.ingest(gpu_ctx, d, cfg, None)
    for k in ("x", "y", "z", "layer", "hit_id", "event"):
        assert np.array_equal(getattr(b, k), getattr(want, k)), k
    r = oracle.run(want, cfg, w.grid(3), 4, n_threads=1)
    _, _, _, _, trk = build_triplets(gpu_ctx, b, cfg, w.n_sectors_z, w.n_sectors_phi)
    assert np.array_equal(trk.hits(), oracle.canonical(r)["tracklets"])
    assert len(trk.hits()) > 0
