"""Event ingest on the CPU: the native decoder of the reference's event files
against the oracle's wire-format reader, decoder error handling, and the
oracle's HitCollection::addEvent restatement on a hand-built event."""
import os

import numpy as np
import pytest

import oracle
import oracle.pb as opb
from pb_util import container, encode_event, event_store, synth_events, _ld, _u, _key
from trax_gb300 import ingest
from trax_gb300.runtime import TraxError

from oracle.ref_build import DEFAULT_REFERENCE  # noqa: E402

TTBAR = os.path.join(DEFAULT_REFERENCE, "plotting", "data", "physics", "hits.ttBar.pb")
COLS = ("run", "lumi", "event_number", "hit_offset", "x", "y", "z", "detector_type", "layer",
        "detector_id", "hit_id", "sim_track_id", "sim_track_pt")


@pytest.fixture(scope="module", autouse=True)
def lib():
    from trax_gb300 import build
    build.build()


def same(d, o):
    for k in COLS:
        assert np.array_equal(getattr(d, k), o[k]), k


@pytest.mark.parametrize("seed,n", [(1, 1), (2, 5), (3, 0)])
def test_decoder_matches_oracle_reader(seed, n):
    evs = synth_events(seed, n)
    for fmt, buf in ((ingest.CONTAINER, container(evs)), (ingest.EVENT_STORE, event_store(evs))):
        d = ingest.decode(buf, fmt)
        same(d, opb.decode(buf, fmt))
        assert d.n_events == n


def test_decoder_threads_agree():
    buf = container(synth_events(4, 7))
    a, b = ingest.decode(buf, n_threads=1), ingest.decode(buf, n_threads=5)
    for k in COLS:
        assert np.array_equal(getattr(a, k), getattr(b, k))


@pytest.mark.skipif(not os.path.exists(TTBAR), reason="reference checkout not present")
def test_decoder_on_reference_ttbar_file():
    buf = open(TTBAR, "rb").read()
    d = ingest.decode(buf)
    same(d, opb.decode(buf))
    assert d.n_events == 10
    assert np.diff(d.hit_offset.astype(np.int64)).tolist()[:3] == [1582, 941, 1088]
    assert set(np.unique(d.layer).tolist()) == {1, 2, 3, 4, 5, 8, 9}


def test_decoder_skips_unknown_fields_and_reads_negative_enum():
    hit = _ld(1, b"\x0d" + b"\x00\x00\x80\x3f" + b"\x15" + b"\x00\x00\x00\x40" + b"\x1d" +
              b"\x00\x00\x40\x40")
    hit += _u(2, -1) + _u(3, 2) + _u(4, 77) + _u(5, 5) + _u(9, 123) + _key(10, 1) + b"\x00" * 8
    ev = _u(1, 1) + _u(2, 2) + _u(3, 3) + _ld(4, hit) + _ld(11, b"junk")
    d = ingest.decode(_ld(1, ev))
    assert d.detector_type.tolist() == [-1] and d.layer.tolist() == [2]
    assert d.x.tolist() == [1.0] and d.z.tolist() == [3.0]
    assert d.sim_track_id.tolist() == [0] and d.sim_track_pt.tolist() == [0.0]


def test_decoder_rejects_bad_input():
    good = container(synth_events(5, 2))
    with pytest.raises(TraxError):
        ingest.decode(good[:-3])
    no_layer = _ld(1, _u(1, 1) + _u(2, 1) + _u(3, 1) + _ld(4, _ld(1, b"\x0d\0\0\0\0\x15\0\0\0\0\x1d\0\0\0\0")
                                                            + _u(2, 0) + _u(4, 1) + _u(5, 1)))
    with pytest.raises(TraxError):
        ingest.decode(no_layer)
    with pytest.raises(TraxError):
        ingest.decode(b"\x07\x00\x00\x00\x02", ingest.EVENT_STORE)


# hand-built event: (track, layer, pt) per hit, min_pt 1, triplet layers 1-2-3
HAND = [(5, 2, 2.0), (3, 1, 2.0), (5, 1, 2.0), (0, 1, 0.0), (3, 2, 2.0), (5, 3, 2.0),
        (3, 3, 2.0), (9, 1, 0.5), (9, 2, 0.5), (9, 3, 0.5), (7, 1, 2.0), (7, 3, 2.0),
        (3, 1, 2.0), (5, 4, 2.0)]


def hand_columns():
    t = np.array([h[0] for h in HAND], np.uint32)
    l = np.array([h[1] for h in HAND], np.uint32)
    p = np.array([h[2] for h in HAND], np.float32)
    return l, t, p, np.array([0, len(HAND)], np.uint64)


# (only_tracks, num_tracks) -> (hit order, layer counts, tracks (id, inner, middle, outer))
HAND_EXPECTED = {
    (1, -1): ([1, 12, 2, 4, 0, 6, 5], [3, 2, 2], [(3, 1, 4, 6), (5, 2, 5, 13)]),
    (0, -1): ([10, 1, 12, 2, 4, 0, 11, 6, 5], [4, 2, 3], [(3, 1, 4, 6), (5, 2, 5, 13)]),
    (1, 1): ([1, 12, 4, 6], [2, 1, 1], [(3, 1, 4, 6)]),
    (0, 1): ([1, 12, 4, 6], [2, 1, 1], [(3, 1, 4, 6)]),
    (1, 0): ([], [0, 0, 0], []),
}


@pytest.mark.parametrize("key", list(HAND_EXPECTED))
def test_oracle_add_event_hand_built(key):
    only, num = key
    l, t, p, off = hand_columns()
    idx, ln, trk, toff = oracle.add_events(l, t, p, off, 1.0, 3, 0b111, only, num)
    want_idx, want_ln, want_trk = HAND_EXPECTED[key]
    assert idx.tolist() == want_idx
    assert ln.reshape(-1).tolist() == want_ln
    assert [tuple(r) for r in trk.tolist()] == want_trk
    assert toff.tolist() == [0, len(want_trk)]


@pytest.mark.skipif(not os.path.exists(TTBAR), reason="reference checkout not present")
def test_oracle_add_event_on_ttbar_selects_findable_tracks():
    d = ingest.decode(open(TTBAR, "rb").read())
    idx, ln, trk, toff = oracle.add_events(d.layer, d.sim_track_id, d.sim_track_pt,
                                           d.hit_offset, 1.0, 4, 0xF)
    # every selected hit belongs to a findable track, on layers 1-4, pT >= 1
    assert (d.sim_track_pt[idx] >= 1.0).all() and (d.layer[idx] <= 4).all()
    for e in range(10):
        ids = set(trk[toff[e]:toff[e + 1], 0].tolist())
        lo, hi = int(d.hit_offset[e]), int(d.hit_offset[e + 1])
        sel = idx[(idx >= lo) & (idx < hi)]
        assert set(d.sim_track_id[sel].tolist()) == ids
        for tid in ids:
            m = (d.sim_track_id[lo:hi] == tid) & (d.sim_track_pt[lo:hi] >= 1.0)
            assert {1, 2, 3, 4} <= set(d.layer[lo:hi][m].tolist())
