"""Operator surface of the reference's seeding chain over the C-ABI.

Names, argument order and meaning follow the reference's classes:
  GridBuilder.run(hits, n_threads, event_supplement, layer_supplement, grid)
      src/algorithms/GridBuilder.h:42 -- sorts `hits` in place, fills `grid`
  PairGeneratorBeamspot.run(hits, geom_supplement, n_threads, layer_triplets, grid)
      src/algorithms/PairGeneratorBeamspot.h:40-41 -- returns a Pairing
  TripletThetaPhiPredictor.run(hits, geom, geom_supplement, dict, n_threads,
                               layer_triplets, grid, pairs)
      src/algorithms/TripletThetaPhiPredictor.h:43-44 -- returns a Pairing
  TripletThetaPhiFilter.run(hits, grid, pairs, triplet_candidates, n_threads,
                            layer_triplets)
      src/algorithms/TripletThetaPhiFilter.h:46-48 -- returns a TrackletCollection
`n_threads` (the OpenCL work-group size) is accepted and ignored: launch
shapes are chosen for the GPU.  `geom` and `dict` are accepted and unused, as
in the reference kernels (TripletThetaPhiPredictor.h:51).  Like the
reference, a stage that returns a collection learns its size on the host
(a synchronisation); the batched Pipeline below does not.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .gen import EventBatch
from .runtime import Context, DeviceBuffer, TraxError, PinnedBuffer

U32 = np.uint32


class EventSupplement:
    """Per event (nHits, offset) -- EventSupplement.h:8-32."""

    def __init__(self, nhits, offset):
        self.nhits = np.ascontiguousarray(nhits, dtype=U32)
        self.offset = np.ascontiguousarray(offset, dtype=U32)

    @property
    def n_events(self):
        return int(self.nhits.size)


class LayerSupplement:
    """Per (event, layer) (nHits, offset within event) -- LayerSupplement.h:7-31."""

    def __init__(self, n_layers, nhits, offset):
        self.n_layers = int(n_layers)
        self.nhits = np.ascontiguousarray(nhits, dtype=U32).reshape(-1)
        self.offset = np.ascontiguousarray(offset, dtype=U32).reshape(-1)


def supplements(batch: EventBatch):
    return (EventSupplement(batch.event_nhits, batch.event_offset),
            LayerSupplement(batch.n_layers, batch.layer_nhits, batch.layer_offset))


class HitCollection:
    """Device-resident SoA hit columns (HitCollection.h:23).

    GridBuilder.run replaces the columns by their cell-sorted copies, as the
    reference replaces its buffers (GridBuilder.cpp:70,151,156-157); the
    sorted copy adds `phi` and `orig` (input position)."""

    COLS = ("x", "y", "z", "layer", "detector_id", "hit_id", "event")

    def __init__(self, ctx: Context, batch: EventBatch):
        self.ctx = ctx
        self.n = batch.n_hits
        self.input = {k: ctx.upload(v) for k, v in zip(self.COLS, batch.columns())}
        self.sorted = None

    def _hits_struct(self):
        d = self.input
        return A.TraxHits(d["x"].ptr, d["y"].ptr, d["z"].ptr, d["layer"].ptr,
                          d["detector_id"].ptr, d["hit_id"].ptr, d["event"].ptr, self.n)

    def _alloc_sorted(self):
        f, u = np.float32, U32
        self.sorted = {k: self.ctx.alloc(max(self.n, 1), t) for k, t in (
            ("x", f), ("y", f), ("z", f), ("phi", f), ("layer", u), ("detector_id", u),
            ("hit_id", u), ("event", u), ("orig", u))}

    def sorted_struct(self):
        s = self.sorted
        if s is None:
            raise TraxError(1, "hits are not grid-sorted yet (run GridBuilder first)")
        return A.TraxSortedHits(s["x"].ptr, s["y"].ptr, s["z"].ptr, s["phi"].ptr, s["layer"].ptr,
                                s["detector_id"].ptr, s["hit_id"].ptr, s["event"].ptr,
                                s["orig"].ptr, self.n)

    def download(self):
        src = self.sorted if self.sorted is not None else self.input
        return {k: b.download(self.n) for k, b in src.items()}


class Grid:
    """Grid (Grid.h:49-68): E*L*(Z+1)(P+1) cell starts, on the device."""

    def __init__(self, ctx: Context, n_events, n_layers, n_sectors_z, n_sectors_phi):
        self.ctx = ctx
        self.config = A.TraxGridCfg(int(n_events), int(n_layers), int(n_sectors_z),
                                    int(n_sectors_phi))
        self.cells = (int(n_sectors_z) + 1) * (int(n_sectors_phi) + 1)
        self.buf = ctx.alloc(max(int(n_events) * int(n_layers) * self.cells, 1))

    def download(self):
        return self.buf.download(self.config.n_events * self.config.n_layers * self.cells)

    def layer_grid(self, layer, event):
        """LayerGrid (Grid.h:93-131): [(Z+1), (P+1)] view for 1-based `layer`."""
        g = self.download().reshape(self.config.n_events, self.config.n_layers,
                                    self.config.n_sectors_z + 1, self.config.n_sectors_phi + 1)
        return g[event, layer - 1]


class Pairing:
    """Pairing (Pairings.h:9-59): uint2 records + per-(event, triplet) offsets."""

    def __init__(self, ctx: Context, capacity: int, n_events: int, n_triplets: int):
        self.ctx = ctx
        self.capacity = int(max(capacity, 1))
        self.n_groups = int(n_events) * int(n_triplets)
        self.records = ctx.alloc(2 * self.capacity)
        self.offsets_buf = ctx.alloc(self.n_groups + 1).zero()
        self.count = None

    def struct(self):
        return A.TraxPairs(self.records.ptr, self.offsets_buf.ptr, self.capacity)

    def get_pairings(self):
        n = self.count if self.count is not None else self.capacity
        return self.records.download(2 * min(n, self.capacity)).reshape(-1, 2)

    def get_pairing_offsets(self):
        return self.offsets_buf.download(self.n_groups + 1)


class TrackletCollection:
    """TrackletCollection (TrackletCollection.h:32-77): hit1/2/3 + offsets."""

    def __init__(self, ctx: Context, capacity: int, n_events: int, n_triplets: int):
        self.ctx = ctx
        self.capacity = int(max(capacity, 1))
        self.n_groups = int(n_events) * int(n_triplets)
        self.cols = [ctx.alloc(self.capacity) for _ in range(3)]
        self.offsets_buf = ctx.alloc(self.n_groups + 1).zero()
        self.connectivity = ctx.alloc(self.capacity).zero()  # TrackletConnectivity item
        self.count = None

    @classmethod
    def from_host(cls, ctx: Context, hits: np.ndarray, connectivity=None):
        """A collection from host (hit1, hit2, hit3) rows, e.g. test tables."""
        hits = np.ascontiguousarray(hits, dtype=U32).reshape(-1, 3)
        t = cls(ctx, max(len(hits), 1), 1, 1)
        for i in range(3):
            if len(hits):
                t.cols[i].upload(hits[:, i])
        if connectivity is not None and len(hits):
            t.connectivity.upload(np.asarray(connectivity, dtype=U32))
        t.count = len(hits)
        return t

    def get_connectivity(self):
        return self.connectivity.download(self.count or 0)

    def struct(self):
        return A.TraxTracklets(self.cols[0].ptr, self.cols[1].ptr, self.cols[2].ptr,
                               self.offsets_buf.ptr, self.capacity)

    def hits(self):
        n = min(self.count or 0, self.capacity)
        return np.stack([c.download(n) for c in self.cols], axis=1) if n else np.zeros((0, 3), U32)

    def get_tracklet_offsets(self):
        return self.offsets_buf.download(self.n_groups + 1)


class _Op:
    def __init__(self, ctx: Context):
        self.ctx = ctx

    def _configure(self, layer_triplets, geom_supplement=None):
        if layer_triplets is not None and layer_triplets is not self.ctx.config:
            self.ctx.configure(layer_triplets)


class GridBuilder(_Op):
    def run(self, hits: HitCollection, n_threads, event_supplement: EventSupplement,
            layer_supplement: LayerSupplement, grid: Grid):
        ctx = self.ctx
        lay = A.TraxLayout(event_supplement.n_events, layer_supplement.n_layers,
                           event_supplement.nhits.ctypes.data, event_supplement.offset.ctypes.data,
                           layer_supplement.nhits.ctypes.data, layer_supplement.offset.ctypes.data)
        if hits.sorted is None:
            hits._alloc_sorted()
        hs = hits._hits_struct()
        out = hits.sorted_struct()
        ctx._check(ctx.lib.trax_grid_build(ctx.h, C.byref(hs), C.byref(lay),
                                           C.byref(grid.config), C.byref(out), grid.buf.ptr))
        return 0


def _grow(ctx, first_cap, make, run):
    """Runs a stage whose output size is only known on the device: if the
    result overflowed the capacity, reallocate to the exact size and rerun."""
    obj = make(first_cap)
    total = run(obj)
    if total > obj.capacity:
        obj = make(total)
        total = run(obj)
    obj.count = total
    return obj


class PairGeneratorBeamspot(_Op):
    def run(self, hits: HitCollection, geom_supplement, n_threads, layer_triplets, grid: Grid,
            capacity=None):
        ctx = self.ctx
        self._configure(layer_triplets)
        T = ctx.config.n_layer_triplets
        sh = hits.sorted_struct()

        def run_once(p: Pairing):
            ctx.reset_counts()
            ps = p.struct()
            ctx._check(ctx.lib.trax_pair_gen(ctx.h, C.byref(sh), grid.buf.ptr, C.byref(grid.config),
                                             C.byref(ps)))
            c = ctx.counts()
            if c["status"] not in (0, 5):
                raise TraxError(c["status"], f"device fault detail {c['error_detail']}")
            self.counts = c
            return c["n_pairs"]

        cap = capacity or max(64 * hits.n, 1024)
        return _grow(ctx, cap, lambda n: Pairing(ctx, n, grid.config.n_events, T), run_once)


class PairGeneratorSector(_Op):
    """PairGeneratorSector::run (PairGeneratorSector.h:38-39, .cpp:5-151):
    every layer-2 hit in the cells within pairSpreadZ / pairSpreadPhi of the
    layer-1 hit's own cell, no cut."""

    def run(self, hits: HitCollection, geom_supplement, n_threads, layer_triplets, grid: Grid,
            capacity=None):
        ctx = self.ctx
        self._configure(layer_triplets)
        T = ctx.config.n_layer_triplets
        sh = hits.sorted_struct()

        def run_once(p: Pairing):
            ctx.reset_counts()
            ps = p.struct()
            ctx._check(ctx.lib.trax_pair_gen_sector(ctx.h, C.byref(sh), grid.buf.ptr,
                                                    C.byref(grid.config), C.byref(ps)))
            c = ctx.counts()
            if c["status"] not in (0, 5):
                raise TraxError(c["status"], f"device fault detail {c['error_detail']}")
            self.counts = c
            return c["n_pairs"]

        cap = capacity or max(256 * hits.n, 1024)
        return _grow(ctx, cap, lambda n: Pairing(ctx, n, grid.config.n_events, T), run_once)


PAIR_GENERATOR_CLASSES = {"beamspot": PairGeneratorBeamspot, "sector": PairGeneratorSector}


class TripletThetaPhiPredictor(_Op):
    def run(self, hits: HitCollection, geom, geom_supplement, dictionary, n_threads,
            layer_triplets, grid: Grid, pairs: Pairing, capacity=None):
        ctx = self.ctx
        self._configure(layer_triplets)
        T = ctx.config.n_layer_triplets
        sh = hits.sorted_struct()

        def run_once(c: Pairing):
            ctx.reset_counts()
            ps, cs = pairs.struct(), c.struct()
            ctx._check(ctx.lib.trax_triplet_predict(ctx.h, C.byref(sh), grid.buf.ptr,
                                                    C.byref(grid.config), C.byref(ps), C.byref(cs)))
            cnt = ctx.counts()
            if cnt["status"] not in (0, 5):
                raise TraxError(cnt["status"], f"device fault detail {cnt['error_detail']}")
            self.counts = cnt
            return cnt["n_candidates"]

        cap = capacity or max(4 * (pairs.count or 0), 1024)
        return _grow(ctx, cap, lambda n: Pairing(ctx, n, grid.config.n_events, T), run_once)


class TripletThetaPhiFilter(_Op):
    def run(self, hits: HitCollection, grid: Grid, pairs: Pairing, triplet_candidates: Pairing,
            n_threads, layer_triplets, capacity=None):
        ctx = self.ctx
        self._configure(layer_triplets)
        T = ctx.config.n_layer_triplets
        sh = hits.sorted_struct()

        def run_once(t: TrackletCollection):
            ctx.reset_counts()
            ps, cs, ts = pairs.struct(), triplet_candidates.struct(), t.struct()
            ctx._check(ctx.lib.trax_triplet_filter(ctx.h, C.byref(sh), C.byref(grid.config),
                                                   C.byref(ps), C.byref(cs), C.byref(ts)))
            cnt = ctx.counts()
            if cnt["status"] not in (0, 5):
                raise TraxError(cnt["status"], f"device fault detail {cnt['error_detail']}")
            self.counts = cnt
            return cnt["n_tracklets"]

        cap = capacity or max(triplet_candidates.count or 0, 1024)
        return _grow(ctx, cap, lambda n: TrackletCollection(ctx, n, grid.config.n_events, T),
                     run_once)


class TripletConnectivity(_Op):
    """TripletConnectivity::run (TripletConnectivity.h:52-54)."""

    def run(self, tracklets_base: TrackletCollection, tracklets_following: TrackletCollection,
            iterate_backwards=False, tight_packing=False):
        ctx = self.ctx
        b, f = tracklets_base.struct(), tracklets_following.struct()
        ctx._check(ctx.lib.trax_triplet_connectivity(
            ctx.h, C.byref(b), tracklets_base.count or 0, tracklets_base.connectivity.ptr,
            C.byref(f), tracklets_following.count or 0, tracklets_following.connectivity.ptr,
            1 if iterate_backwards else 0, 1 if tight_packing else 0))


def build_triplets(ctx: Context, batch: EventBatch, cfg: A.TraxConfig, n_sectors_z,
                   n_sectors_phi, n_threads=256, pair_generator="beamspot"):
    """The reference's call order (TripletBuilder.cpp:240-263) on one group."""
    ctx.configure(cfg)
    hits = HitCollection(ctx, batch)
    es, ls = supplements(batch)
    grid = Grid(ctx, batch.n_events, batch.n_layers, n_sectors_z, n_sectors_phi)
    GridBuilder(ctx).run(hits, n_threads, es, ls, grid)
    pairs = PAIR_GENERATOR_CLASSES[pair_generator](ctx).run(hits, cfg, n_threads, cfg, grid)
    cands = TripletThetaPhiPredictor(ctx).run(hits, None, cfg, None, n_threads, cfg, grid, pairs)
    trk = TripletThetaPhiFilter(ctx).run(hits, grid, pairs, cands, n_threads, cfg)
    return hits, grid, pairs, cands, trk


def _host_cols(b: EventBatch):
    """The batch's columns, contiguous; a column given as None (the detector
    and hit ids, which the batched calls do not read) stays None."""
    return [None if c is None else np.ascontiguousarray(c) for c in b.columns()]


def _col_ptrs(cols):
    return [None if c is None else c.ctypes.data for c in cols]


class Pipeline:
    """Batched form: reserved buffers, one CUDA graph per run, no host sync
    inside the chain (trax_reserve / trax_seed_batch)."""

    def __init__(self, ctx: Context, cfg: A.TraxConfig, grid: A.TraxGridCfg, max_events,
                 max_hits, max_pairs, max_candidates, max_tracklets, pair_generator="beamspot",
                 tuning_by_class=None):
        """tuning_by_class: density class -> tuning (autotune.autotune()'s
        per-class "tuning"); each batch then runs with its class's tuning,
        which changes speed only."""
        self.ctx = ctx
        ctx.configure(cfg)
        ctx.set_pair_generator(pair_generator)
        self.tuning_by_class = tuning_by_class
        self._tuning = None
        self.n_triplets = cfg.n_layer_triplets
        self.max_tracklets = int(max_tracklets)
        self.n_layers = grid.n_layers
        ctx._check(ctx.lib.trax_reserve(ctx.h, int(max_events), grid.n_layers, int(max_hits),
                                        C.byref(grid), int(max_pairs), int(max_candidates),
                                        int(max_tracklets)))
        self._keep = []
        # pinned result buffers, reused by every seed() call
        cap = self.max_tracklets
        self._out = [PinnedBuffer(ctx, 4 * cap, U32) for _ in range(3)]
        self._off_len = int(max_events) * self.n_triplets + 1
        self._off = PinnedBuffer(ctx, 4 * self._off_len, U32)
        # streaming (submit / wait): two slots, result buffers made on first use
        self._stream_out = [None, None]
        self._inflight = {}

    def _apply_tuning(self, b: EventBatch):
        from .autotune import tuning_for
        t = tuning_for(self.tuning_by_class, b.n_hits / max(1, b.n_events))
        if t is not None and t != self._tuning:
            self.ctx.set_tuning(*t)
            self._tuning = t

    def _batch_struct(self, b: EventBatch):
        self._apply_tuning(b)
        cols = _host_cols(b)
        ln = np.ascontiguousarray(b.layer_nhits.reshape(-1), dtype=U32)
        self._keep = cols + [ln]
        return A.TraxEventBatch(b.n_events, b.n_layers, b.n_hits, *_col_ptrs(cols), ln.ctypes.data)

    def seed(self, b: EventBatch, input_indices=False, copy=True):
        """Host arrays in, tracklets out (synchronous).  With copy=False the
        returned arrays are views of pinned buffers that the next call
        overwrites."""
        bs = self._batch_struct(b)
        cap = self.max_tracklets
        h = [o.array for o in self._out]
        r = A.TraxBatchResult(self._out[0].ptr, self._out[1].ptr, self._out[2].ptr,
                              self._off.ptr, cap, 1 if input_indices else 0, 0, A.TraxCounts())
        self.ctx._check(self.ctx.lib.trax_seed_batch(self.ctx.h, C.byref(bs), C.byref(r)))
        n = r.n_tracklets
        off = self._off.array[: b.n_events * self.n_triplets + 1]
        if not copy:
            return [x[:n] for x in h], off, r.counts.as_dict()
        return np.stack([x[:n] for x in h], axis=1), off.copy(), r.counts.as_dict()

    def submit(self, b: EventBatch, input_indices=False):
        """Streaming form (trax_submit_batch): queues `b` and returns a ticket
        at once; two batches may be in flight, each with its own pinned
        result buffers.  `b`'s arrays must stay unchanged until wait()."""
        if not self._inflight:  # never change the tuning under a batch in flight
            self._apply_tuning(b)
        busy = {v[3] for v in self._inflight.values()}
        free = [k for k in (0, 1) if k not in busy]
        if not free:
            raise RuntimeError("two batches in flight: wait for the older one first")
        k = free[0]
        if self._stream_out[k] is None:
            cap = self.max_tracklets
            self._stream_out[k] = ([PinnedBuffer(self.ctx, 4 * cap, U32) for _ in range(3)],
                                   PinnedBuffer(self.ctx, 4 * self._off_len, U32))
        outs, off = self._stream_out[k]
        cols = _host_cols(b)
        ln = np.ascontiguousarray(b.layer_nhits.reshape(-1), dtype=U32)
        bs = A.TraxEventBatch(b.n_events, b.n_layers, b.n_hits, *_col_ptrs(cols), ln.ctypes.data)
        r = A.TraxBatchResult(outs[0].ptr, outs[1].ptr, outs[2].ptr, off.ptr, self.max_tracklets,
                              1 if input_indices else 0, 0, A.TraxCounts())
        t = C.c_uint32()
        self.ctx._check(self.ctx.lib.trax_submit_batch(self.ctx.h, C.byref(bs), C.byref(r),
                                                       C.byref(t)))
        self._inflight[t.value] = (r, cols + [ln], b.n_events, k)
        return t.value

    def wait(self, ticket, copy=True):
        """Waits for a submitted batch; returns (tracklets, offsets, counts)
        like seed() (copy=False: views of the batch's pinned buffers, valid
        until the next submit)."""
        if ticket not in self._inflight:
            raise RuntimeError(f"no batch in flight with ticket {ticket}")
        r, _, n_events, k = self._inflight.pop(ticket)
        self.ctx._check(self.ctx.lib.trax_wait_batch(self.ctx.h, ticket, C.byref(r)))
        outs, off = self._stream_out[k]
        n = r.n_tracklets
        h = [o.array[:n] for o in outs]
        o = off.array[: n_events * self.n_triplets + 1]
        if not copy:
            return h, o, r.counts.as_dict()
        return np.stack(h, axis=1), o.copy(), r.counts.as_dict()

    def stage(self, b: EventBatch):
        bs = self._batch_struct(b)
        self.ctx._check(self.ctx.lib.trax_stage_batch(self.ctx.h, C.byref(bs)))

    def run_staged(self):
        self.ctx._check(self.ctx.lib.trax_run_staged(self.ctx.h))
