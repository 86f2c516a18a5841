"""Event ingest: the reference's event files into HitCollection batches.

Mirrors the reference's loading path (EventLoader.h:15-111,
TripletBuilder.cpp:112-214): decode a PEventContainer file or an event
store (native decoder, trax_pb_decode), then HitCollection::addEvent for a
batch of events (GPU, trax_ingest), with the detector geometry
(DetectorGeometry / GeometrySupplement from configs/detectorRadius.dat and
radiusDictionary.dat, TripletBuilder.cpp:100-141).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from .gen import EventBatch
from .runtime import Context, TraxError, load_library

CONTAINER, EVENT_STORE = A.PB_CONTAINER, A.PB_EVENT_STORE
U32 = np.uint32


@dataclass
class DecodedEvents:
    """PEvent / PHit fields as flat columns (trax_pb_events)."""
    run: np.ndarray
    lumi: np.ndarray
    event_number: np.ndarray
    hit_offset: np.ndarray
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    detector_type: np.ndarray
    layer: np.ndarray
    detector_id: np.ndarray
    hit_id: np.ndarray
    sim_track_id: np.ndarray
    sim_track_pt: np.ndarray

    @property
    def n_events(self):
        return len(self.run)

    @property
    def n_hits(self):
        return len(self.x)

    def select(self, first, count, repeat=False):
        """Events [first, first + count), or event `first` repeated `count`
        times (RepeatedEventLoader, EventLoader.h:67-111)."""
        idx = [first] * count if repeat else list(range(first, min(first + count, self.n_events)))
        parts = [(int(self.hit_offset[e]), int(self.hit_offset[e + 1])) for e in idx]
        cat = lambda a: np.concatenate([a[lo:hi] for lo, hi in parts]) if parts else a[:0]
        off = np.zeros(len(idx) + 1, np.uint64)
        off[1:] = np.cumsum([hi - lo for lo, hi in parts])
        ev = lambda a: a[idx] if idx else a[:0]
        return DecodedEvents(ev(self.run), ev(self.lumi), ev(self.event_number), off,
                             *(cat(getattr(self, k)) for k in (
                                 "x", "y", "z", "detector_type", "layer", "detector_id", "hit_id",
                                 "sim_track_id", "sim_track_pt")))


def decode(buf: bytes, fmt=CONTAINER, n_threads=0) -> DecodedEvents:
    L = load_library()
    raw = np.frombuffer(buf, np.uint8)
    ptr = raw.ctypes.data if raw.size else None
    ne, nh = C.c_uint32(0), C.c_uint64(0)
    st = L.trax_pb_scan(ptr, raw.size, fmt, C.byref(ne), C.byref(nh))
    if st:
        raise TraxError(st, L.trax_pb_error().decode())
    E, N = ne.value, nh.value
    d = DecodedEvents(np.zeros(E, np.uint64), np.zeros(E, np.uint64), np.zeros(E, np.uint64),
                      np.zeros(E + 1, np.uint64), np.zeros(N, np.float32), np.zeros(N, np.float32),
                      np.zeros(N, np.float32), np.zeros(N, np.int32), np.zeros(N, U32),
                      np.zeros(N, U32), np.zeros(N, np.uint64), np.zeros(N, U32),
                      np.zeros(N, np.float32))
    s = A.TraxPbEvents(E, N, *(getattr(d, k).ctypes.data for k in (
        "run", "lumi", "event_number", "hit_offset", "x", "y", "z", "detector_type", "layer",
        "detector_id", "hit_id", "sim_track_id", "sim_track_pt")))
    st = L.trax_pb_decode(ptr, raw.size, fmt, C.byref(s), n_threads)
    if st:
        raise TraxError(st, L.trax_pb_error().decode())
    return d


def load_file(path, fmt=CONTAINER) -> DecodedEvents:
    with open(path, "rb") as f:
        return decode(f.read(), fmt)


@dataclass
class Geometry:
    """DetectorGeometry (detId -> layer, file order) and the per-layer
    radius range of GeometrySupplement (index layer - 1)."""
    det_ids: np.ndarray
    det_layer: np.ndarray
    min_radius: np.ndarray
    max_radius: np.ndarray


def load_geometry(detector_radius_path, radius_dictionary_path, n_layers=13) -> Geometry:
    """configs/detectorRadius.dat rows (detId, dictEntry, layer) and
    radiusDictionary.dat rows (entry, radius), as TripletBuilder.cpp:100-141
    reads them: the radius range of layer l is the min / max dictionary
    radius over its modules (10000 / 0 when it has none)."""
    radius = {}
    for line in open(radius_dictionary_path):
        line = line.strip()
        if line:
            k, r = line.split(",")[:2]
            radius[len(radius)] = float(r)
    ids, layers = [], []
    rmin = np.full(n_layers, 10000.0, np.float32)
    rmax = np.zeros(n_layers, np.float32)
    for line in open(detector_radius_path):
        line = line.strip()
        if not line:
            continue
        det, entry, layer = (int(v) for v in line.split(",")[:3])
        ids.append(det)
        layers.append(layer)
        r = np.float32(radius[entry])
        if 1 <= layer <= n_layers:
            rmax[layer - 1] = max(rmax[layer - 1], r)
            rmin[layer - 1] = min(rmin[layer - 1], r)
    return Geometry(np.array(ids, U32), np.array(layers, U32), rmin, rmax)


def used_layers(cfg: A.TraxConfig):
    """(max layer, bit mask) of the layers the triplets use
    (HitCollection.cpp:26-35)."""
    mask, top = 0, 0
    for i in range(cfg.n_layer_triplets):
        t = cfg.triplets[i]
        for l in (t.layer1, t.layer2, t.layer3):
            mask |= 1 << (l - 1)
        top = max(top, t.layer3)
    return top, mask


@dataclass
class TrackList:
    """Findable tracks per event (HitCollection::tTrackList): track id and
    the raw hit indices of its first, middle and last hit in layer order."""
    track_id: np.ndarray
    inner: np.ndarray
    middle: np.ndarray
    outer: np.ndarray
    offsets: np.ndarray


def ingest(ctx: Context, ev: DecodedEvents, cfg: A.TraxConfig, det_ids=None,
           num_tracks=-1, only_tracks=True):
    """HitCollection::addEvent for every event on the GPU.  Returns the
    EventBatch (host copy of the HitCollection and supplements) and the
    findable-track list."""
    E, N = ev.n_events, ev.n_hits
    max_layer, mask = used_layers(cfg)

    def dev(a, dt):
        a = np.ascontiguousarray(a, dt)
        return ctx.upload(a if a.size else np.zeros(1, dt))

    cols = [dev(ev.x, np.float32), dev(ev.y, np.float32), dev(ev.z, np.float32),
            dev(ev.layer, U32), dev(ev.detector_id, U32), dev(ev.sim_track_id, U32),
            dev(ev.sim_track_pt, np.float32), dev(ev.hit_offset.astype(U32), U32)]
    raw = A.TraxRawHits(*(c.ptr for c in cols), E, N)
    icfg = A.TraxIngestCfg(cfg.min_pt, max_layer, mask, 1 if only_tracks else 0, num_tracks)
    ids = np.ascontiguousarray(det_ids if det_ids is not None else np.zeros(0), U32)
    d_ids = dev(ids, U32) if ids.size else None
    cap = max(N, 1)
    out_cols = [ctx.alloc(cap, np.float32) for _ in range(3)] + [ctx.alloc(cap, U32) for _ in range(4)]
    out = A.TraxHitsOut(*(c.ptr for c in out_cols), cap)
    ln = ctx.alloc(max(E * max_layer, 1), U32)
    tcols = [ctx.alloc(cap, U32) for _ in range(4)]
    toff = ctx.alloc(E + 1, U32)
    tl = A.TraxTrackList(*(c.ptr for c in tcols), toff.ptr, cap)
    nh, nt = C.c_uint32(0), C.c_uint32(0)
    ctx._check(ctx.lib.trax_ingest(ctx.h, C.byref(raw), C.byref(icfg),
                                   d_ids.ptr if d_ids is not None else None, ids.size,
                                   C.byref(out), ln.ptr, C.byref(tl), C.byref(nh), C.byref(nt)))
    n, t = nh.value, nt.value
    h = [c.download(n) for c in out_cols]
    batch = EventBatch(h[0], h[1], h[2], h[3], h[4], h[5], h[6],
                       ln.download(E * max_layer).reshape(E, max_layer))
    tracks = TrackList(*(c.download(t) for c in tcols), toff.download(E + 1))
    return batch, tracks
