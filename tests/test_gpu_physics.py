"""GPU physics evaluation (trax_physics_eval) against the oracle's
PhysicsRecord::fillData restatement, on events that went file bytes ->
decode -> GPU addEvent -> GPU seeding."""
import numpy as np
import pytest

import oracle
from pb_util import container, events_from_batch
from test_physics import Rec
from trax_gb300 import gen, ingest, load_library
from trax_gb300.ops import build_triplets
from trax_gb300.physics import PhysicsRecords

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,n_ev,only", [("multimuon-1000trk", 3, True),
                                            ("pileup50-batch100", 2, True),
                                            ("multimuon-1000trk", 2, False)])
def test_gpu_physics_matches_oracle(gpu_ctx, name, n_ev, only):
    w = gen.WORKLOADS[name]
    src = gen.generate_batch(w, n_ev)
    pt = lambda t: 0.5 if t % 9 == 0 else 3.0
    d = ingest.decode(container(events_from_batch(src, pt)))
    cfg = w.config()
    b, tracks = ingest.ingest(gpu_ctx, d, cfg, None, only_tracks=only)
    hits, _, _, _, trk = build_triplets(gpu_ctx, b, cfg, w.n_sectors_z, w.n_sectors_phi)
    T = cfg.n_layer_triplets
    rec = PhysicsRecords(gpu_ctx)
    counts, cat = rec.evaluate(hits, trk, n_ev, T, tracks, d)

    srt = hits.download()
    toff = trk.get_tracklet_offsets()
    mc = np.stack([tracks.track_id, tracks.inner, tracks.middle, tracks.outer], axis=1)
    ph = oracle.physics(srt["hit_id"], srt["x"], srt["y"], srt["z"], trk.hits(), toff, n_ev, T,
                        (mc, tracks.offsets), d.x, d.y, d.z)
    assert np.array_equal(counts, ph["counts"])
    assert np.array_equal(cat, ph["cat"])
    assert counts[:, 1].sum() > 0 and counts[:, 0].sum() > 0

    ref = Rec(load_library())
    M = len(mc)
    for e in range(n_ev):
        for lt in range(T):
            g = e * T + lt
            t0, t1 = int(toff[g]), int(toff[g + 1])
            ks = [lt * M + k for k in range(int(tracks.offsets[e]), int(tracks.offsets[e + 1]))
                  if ph["missed"][lt * M + k]]
            ref.add(e, lt, ph["counts"][g], ph["cat"][t0:t1], ph["eta_bin"][t0:t1],
                    ph["pt_bin"][t0:t1], ph["miss_eta_bin"][ks], ph["miss_pt_bin"][ks])
    assert rec.csv() == ref.text()
    for lt in range(T + 2):
        if lt == T:
            continue
        for which, code in (("eta", 1), ("pt", 2)):
            assert rec.histogram_csv(which, lt) == ref.text(code, lt)
