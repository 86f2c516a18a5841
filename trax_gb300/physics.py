"""Physics evaluation: PhysicsRecords (PhysicsRecord.h:94-186) over the GPU
pass trax_physics_eval (PhysicsRecord::fillData for every (event, layer
triplet) of a batch)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .ingest import DecodedEvents, TrackList
from .ops import HitCollection, TrackletCollection
from .runtime import Context, TraxError

COUNT_FIELDS = ("tracklets", "valid", "clones", "fake", "misc", "missed", "findable")


class PhysicsRecords:
    """Records merged per layer triplet; csv() is PhysicsRecords::csvDump,
    histogram_csv() the eta_<lt>.csv / pt_<lt>.csv files it writes."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        ctx._check(self.lib.trax_physics_create(C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.trax_physics_destroy(self.h)
            self.h = None

    def evaluate(self, hits: HitCollection, trk: TrackletCollection, n_events, n_lt,
                 tracks: TrackList, decoded: DecodedEvents):
        """Adds the batch's records; returns (counts [E*T] dicts as an array of
        shape (E*T, 7), per-tracklet categories)."""
        ctx = self.ctx
        up = lambda a, dt: ctx.upload(np.ascontiguousarray(a, dt) if len(a) else np.zeros(1, dt))
        cols = [up(tracks.track_id, np.uint32), up(tracks.inner, np.uint32),
                up(tracks.middle, np.uint32), up(tracks.outer, np.uint32),
                up(tracks.offsets, np.uint32)]
        tl = A.TraxTrackList(*(c.ptr for c in cols), max(len(tracks.track_id), 1))
        raw = [up(decoded.x, np.float32), up(decoded.y, np.float32), up(decoded.z, np.float32)]
        G = n_events * n_lt
        counts = np.zeros((max(G, 1), 7), np.uint32)
        n_trk = int(trk.get_tracklet_offsets()[-1]) if G else 0
        cat = np.zeros(max(n_trk, 1), np.uint8)
        sh, ts = hits.sorted_struct(), trk.struct()
        ctx._check(self.lib.trax_physics_eval(ctx.h, self.h, C.byref(sh), C.byref(ts), n_events,
                                              n_lt, C.byref(tl), raw[0].ptr, raw[1].ptr,
                                              raw[2].ptr, counts.ctypes.data, cat.ctypes.data))
        return counts[:G], cat[:n_trk]

    @property
    def n_records(self):
        return int(self.lib.trax_physics_n_records(self.h))

    def _text(self, what, lt=0):
        n = C.c_size_t(0)
        st = self.lib.trax_physics_csv(self.h, what, lt, None, 0, C.byref(n))
        if st:
            raise TraxError(st, "no such record")
        buf = C.create_string_buffer(n.value + 1)
        self.ctx._check(self.lib.trax_physics_csv(self.h, what, lt, buf, n.value + 1, C.byref(n)))
        return buf.value.decode()

    def csv(self):
        return self._text(0)

    def histogram_csv(self, which, layer_triplet):
        """which: "eta" or "pt"; layer_triplet: the record, or n_records + 1
        for the merged total."""
        return self._text(1 if which == "eta" else 2, layer_triplet)
