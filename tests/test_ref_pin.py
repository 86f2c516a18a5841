"""The oracle pinned to the reference: the reference's own OpenCL kernels,
compiled for the host (oracle/ref_build.py) and run through its host chain
(oracle/ref_host.cpp), against the CPU restatement (trax_oracle.c) on the
same seeded inputs.  Every stage's output must be equal element for element:
the grid, all seven sorted hit columns (float bits), the pair slots and pair
offsets, the candidate slots and candidate offsets, the tracklets and their
offsets, and the slot totals -- at the reference's work-group sizes, for
every kernel variant the reference picks by local memory size, and for both
pair generators.

The library needs the reference tree to build; without it (and without a
library built earlier) the module is skipped.
"""
import numpy as np
import pytest

import oracle
from oracle import ref
from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg

pytestmark = pytest.mark.skipif(not ref.available(),
                                reason="reference tree absent: oracle/_ref cannot be built")

COMPARED = ("sorted_x", "sorted_y", "sorted_z", "sorted_layer", "sorted_det", "sorted_hitid",
            "sorted_event", "grid", "pairs", "pair_valid", "pair_offsets", "cands", "cand_valid",
            "cand_offsets", "trk_h1", "trk_h2", "trk_h3", "trk_offsets")
SLOT_STATS = ("status", "pair_slots", "pairs", "cand_slots", "cands", "tracklets")


def assert_same(o, r):
    for k in COMPARED:
        a, b = o[k], r[k]
        assert a.shape == b.shape, (k, a.shape, b.shape)
        if k in ("pairs", "cands"):
            valid = o["pair_valid" if k == "pairs" else "cand_valid"].astype(bool)
            assert np.array_equal(a[valid], b[valid]), k
        else:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), k
    for k in SLOT_STATS:
        assert o["stats"][k] == r["stats"][k], (k, o["stats"], r["stats"])


def batch_for(name, n_events):
    w = gen.WORKLOADS[name]
    return w, gen.generate_batch(w, n_events), w.config(), w.grid(n_events)


@pytest.mark.parametrize("name,n_events,n_threads", [
    ("single-muon-100trk", 3, 1),
    ("single-muon-100trk", 3, 256),
    ("single-muon-100trk", 3, 8),
    ("multimuon-1000trk", 2, 1),
    ("multimuon-1000trk", 2, 256),
    ("pileup50-batch100", 4, 1),
    ("pileup50-batch100", 3, 256),
    ("stream-pileup-u200", 3, 64),
])
def test_oracle_equals_reference_kernels(name, n_events, n_threads):
    w, b, cfg, g = batch_for(name, n_events)
    o = oracle.run(b, cfg, g, 4, n_threads=n_threads)
    r = ref.run(b, cfg, g, 4, n_threads=n_threads)
    assert r["stats"]["status"] == 0
    assert o["stats"]["tracklets"] > 0
    assert_same(o, r)


def test_pileup200_with_an_unwritten_candidate_slot():
    """Two pile-up-200 events leave one candidate slot unwritten (the store
    window accepts fewer than the count window counted): both sides define
    that slot as never accepted."""
    w, b, cfg, g = batch_for("pileup200", 2)
    o = oracle.run(b, cfg, g, 4, n_threads=1)
    r = ref.run(b, cfg, g, 4, n_threads=1)
    assert o["stats"]["cands"] < o["stats"]["cand_slots"]
    assert_same(o, r)


@pytest.mark.parametrize("variant", [
    ref.GRID_NO_LOCAL_COUNT,
    ref.GRID_STORE_WRITTEN_LOCAL,
    ref.GRID_STORE_NO_LOCAL,
    ref.PAIR_NO_LOCAL_COUNT,
    ref.GRID_NO_LOCAL_COUNT | ref.GRID_STORE_NO_LOCAL | ref.PAIR_NO_LOCAL_COUNT,
])
def test_every_kernel_variant(variant):
    w, b, cfg, g = batch_for("multimuon-1000trk", 1)
    o = oracle.run(b, cfg, g, 4, n_threads=32)
    r = ref.run(b, cfg, g, 4, n_threads=32, variant=variant)
    assert_same(o, r)


@pytest.mark.parametrize("name,n_events,n_threads", [
    ("single-muon-100trk", 3, 1), ("single-muon-100trk", 2, 64), ("multimuon-1000trk", 1, 256)])
def test_sector_pair_generator(name, n_events, n_threads):
    w, b, cfg, g = batch_for(name, n_events)
    o = oracle.run(b, cfg, g, 4, n_threads=n_threads, pair_gen="sector")
    r = ref.run(b, cfg, g, 4, n_threads=n_threads, pair_gen="sector")
    assert_same(o, r)


@pytest.mark.parametrize("zp", [(8, 16), (64, 128), (64, 64), (256, 192)])
def test_other_grids(zp):
    """Grid granularities the autotuner searches."""
    w, b, cfg, _ = batch_for("multimuon-1000trk", 1)
    g = TraxGridCfg(1, w.n_layers, zp[0], zp[1])
    o = oracle.run(b, cfg, g, 4, n_threads=64)
    r = ref.run(b, cfg, g, 4, n_threads=64)
    assert_same(o, r)


def test_single_cell_grid_double_visits():
    """On a 1 x 1 grid every phi window covers the whole row, so pairCount
    visits cells twice: it counts more slots than pairStore writes (the
    count hazard of PairGeneratorBeamspot.h:216-226).  Slot totals, written
    pairs and their order agree; the reference would then read the unwritten
    slots, so its chain stops there."""
    w, b, cfg, _ = batch_for("multimuon-1000trk", 1)
    g = TraxGridCfg(1, w.n_layers, 1, 1)
    o = oracle.run(b, cfg, g, 2, n_threads=64)
    r = ref.run(b, cfg, g, 2, n_threads=64)
    assert o["stats"]["pairs"] < o["stats"]["pair_slots"]
    assert r["stats"]["status"] == 2
    for k in ("grid", "pairs", "pair_valid", "pair_offsets"):
        a, c = o[k], r[k]
        if k == "pairs":
            a, c = a[o["pair_valid"].astype(bool)], c[o["pair_valid"].astype(bool)]
        assert np.array_equal(a, c), k
    assert o["stats"]["pair_slots"] == r["stats"]["pair_slots"]
    assert o["stats"]["pairs"] == r["stats"]["pairs"]


def test_racy_grid_store_same_cells():
    """With many work-items per (event, layer) the reference's within-cell
    order is a race (GridBuilder.h:243-244); the grid and every cell's set
    of hits still equal the restatement's."""
    w, b, cfg, g = batch_for("multimuon-1000trk", 1)
    b.detector_id = np.arange(b.n_hits, dtype=np.uint32)
    o = oracle.run(b, cfg, g, 1, n_threads=64)
    r = ref.run(b, cfg, g, 1, n_threads=64, grid_threads=64)
    assert np.array_equal(o["grid"], r["grid"])
    starts = np.append(o["grid"], b.n_hits)
    cuts = np.unique(starts)
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        assert sorted(o["sorted_orig"][lo:hi]) == sorted(r["sorted_det"][lo:hi])


def test_empty_layers_and_events():
    """Events whose inner, middle or outer layer is empty, and an event with
    no hits at all."""
    w, b, cfg, g = batch_for("single-muon-100trk", 4)
    keep = np.ones(b.n_hits, bool)
    eo = b.event_offset
    lo, ln = b.layer_offset, b.layer_nhits
    for e, layer in ((0, 0), (1, 1), (2, 2)):
        s = eo[e] + lo[e, layer]
        keep[s:s + ln[e, layer]] = False
    keep[eo[3]:eo[3] + ln[3].sum()] = False
    nh = np.zeros_like(b.layer_nhits)
    np.add.at(nh, (b.event[keep], b.layer[keep] - 1), 1)
    b2 = gen.EventBatch(b.x[keep], b.y[keep], b.z[keep], b.layer[keep], b.detector_id[keep],
                        b.hit_id[keep], b.event[keep], nh)
    assert (nh == 0).sum() >= 6
    o = oracle.run(b2, cfg, g, 4, n_threads=16)
    r = ref.run(b2, cfg, g, 4, n_threads=16)
    assert_same(o, r)


def test_ttbar_events_with_the_reference_configuration():
    """The reference's own ttbar events (hits.ttBar.pb), CMS layer radii and
    cut table, through both chains: real detector data, four layer
    triplets, the ttBar.reco.conf grid of 50 x 8 cells."""
    import os
    from test_physics import TTBAR, load_reference_config
    from trax_gb300 import ingest
    from trax_gb300._abi import make_config
    if not os.path.exists(TTBAR):
        pytest.skip("reference event file absent")
    from trax_gb300 import build
    build.build()
    rows, geo = load_reference_config()
    cfg = make_config(rows, geo.min_radius, geo.max_radius, 1.0)
    d = ingest.decode(open(TTBAR, "rb").read())
    ml, mask = ingest.used_layers(cfg)
    idx, ln, trk, toff = oracle.add_events(d.layer, d.sim_track_id, d.sim_track_pt,
                                           d.hit_offset, 1.0, ml, mask)
    ev = np.repeat(np.arange(d.n_events, dtype=np.uint32), ln.sum(axis=1).astype(np.int64))
    b = gen.EventBatch(d.x[idx], d.y[idx], d.z[idx], d.layer[idx], d.detector_id[idx],
                       d.sim_track_id[idx], ev, ln)
    g = TraxGridCfg(d.n_events, ml, 50, 8)
    o = oracle.run(b, cfg, g, 4, n_threads=256)
    r = ref.run(b, cfg, g, 4, n_threads=256)
    assert o["stats"]["tracklets"] > 0
    assert_same(o, r)
