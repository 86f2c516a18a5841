"""Writes events in the reference's file layouts (Event.proto:1-38;
PEventContainer message, or the event store of PEventStore.h:25-80) and
synthesises events with the features addEvent selects on: sparse track ids,
pT below and above the cut, missing layers, repeated layers, layers beyond
the triplets' range, unassociated (track 0) hits without pT."""
import struct

import numpy as np


def _varint(v):
    v &= (1 << 64) - 1
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _key(f, w):
    return _varint((f << 3) | w)


def _ld(f, payload):
    return _key(f, 2) + _varint(len(payload)) + payload


def _f32(f, v):
    return _key(f, 5) + struct.pack("<f", float(v))


def _u(f, v):
    return _key(f, 0) + _varint(int(v))


def encode_hit(x, y, z, dtype, layer, det, hit_id, track=None, pt=None):
    pos = _f32(1, x) + _f32(2, y) + _f32(3, z)
    b = _ld(1, pos) + _u(2, dtype) + _u(3, layer) + _u(4, det) + _u(5, hit_id)
    if track is not None:
        b += _u(6, track)
    if pt is not None:
        b += _f32(7, pt)
    return b


def encode_event(run, lumi, number, hits):
    b = _u(1, run) + _u(2, lumi) + _u(3, number)
    return b + b"".join(_ld(4, encode_hit(*h)) for h in hits)


def container(events):
    return b"".join(_ld(1, encode_event(*e)) for e in events)


def event_store(events):
    out = struct.pack("<I", len(events))
    for e in events:
        p = encode_event(*e)
        out += _varint(1) + _varint(len(p)) + p
    return out


def synth_events(seed, n_events, n_tracks=60, layers=(1, 2, 3, 4, 5, 8, 9), det_ids=None):
    """Events as (run, lumi, number, hits) with hits (x, y, z, type, layer,
    det, hit_id, track, pt)."""
    rng = np.random.default_rng(seed)
    det_ids = np.arange(1000, 1400, dtype=np.uint32) if det_ids is None else det_ids
    events = []
    for e in range(n_events):
        hits = []
        ids = rng.choice(1 << 22, size=rng.poisson(n_tracks) + 1, replace=False) + 1
        for t in ids:
            pt = float(1.0 / (1 / 0.3 - rng.uniform() * (1 / 0.3 - 1 / 50)))
            have = [l for l in layers if rng.uniform() > 0.12]
            if rng.uniform() < 0.2 and have:  # overlapping modules: a repeated layer
                have.append(have[rng.integers(len(have))])
            rng.shuffle(have)
            for l in have:
                r = 3.0 * l + rng.normal(0, 0.1)
                ph = rng.uniform(-np.pi, np.pi)
                hits.append((r * np.cos(ph), r * np.sin(ph), rng.uniform(-25, 25), 0, l,
                             int(rng.choice(det_ids)) if rng.uniform() < 0.95 else 77,
                             len(hits), int(t), pt))
        for _ in range(rng.poisson(n_tracks // 2)):
            l = int(rng.choice(layers))
            r = 3.0 * l
            ph = rng.uniform(-np.pi, np.pi)
            hits.append((r * np.cos(ph), r * np.sin(ph), rng.uniform(-25, 25), 0, l,
                         int(rng.choice(det_ids)), len(hits), None, None))
        order = rng.permutation(len(hits))
        events.append((1, 7, 900 + e, [hits[i] for i in order]))
    return events


def events_from_batch(b, pt_of_track):
    """PEvents from a generated EventBatch (hit_id holds the track id, 0 for
    noise); pT per track from pt_of_track(id)."""
    events = []
    for e in range(b.n_events):
        lo, hi = int(b.event_offset[e]), int(b.event_offset[e]) + int(b.event_nhits[e])
        hits = []
        for i in range(lo, hi):
            t = int(b.hit_id[i])
            hits.append((float(b.x[i]), float(b.y[i]), float(b.z[i]), 0, int(b.layer[i]),
                         int(b.detector_id[i]), i - lo, t if t else None,
                         pt_of_track(t) if t else None))
        events.append((1, 1, e, hits))
    return events
