"""ctypes mirror of the POD types in include/trax.h."""
from __future__ import annotations

import ctypes as C

MAX_LAYER_TRIPLETS = 16
MAX_LAYERS = 16

TRAX_OK = 0
PAIR_GENERATORS = {"beamspot": 0, "sector": 1}
STATUS_NAMES = {
    0: "TRAX_OK", 1: "TRAX_ERR_BAD_ARG", 2: "TRAX_ERR_OOM", 3: "TRAX_ERR_TIMEOUT",
    4: "TRAX_ERR_DEVICE", 5: "TRAX_ERR_CAPACITY", 6: "TRAX_ERR_BAD_INPUT",
    7: "TRAX_ERR_NO_DEVICE",
}


class TraxGridCfg(C.Structure):
    _fields_ = [("n_events", C.c_uint32), ("n_layers", C.c_uint32),
                ("n_sectors_z", C.c_uint32), ("n_sectors_phi", C.c_uint32)]


class TraxLayerTriplet(C.Structure):
    _fields_ = [("layer1", C.c_uint32), ("layer2", C.c_uint32), ("layer3", C.c_uint32),
                ("dtheta_cut", C.c_float), ("sigma_z", C.c_float), ("dphi_cut", C.c_float),
                ("sigma_phi", C.c_float), ("tip_cut", C.c_float),
                ("pair_spread_z", C.c_uint32), ("z0", C.c_float),
                ("pair_spread_phi", C.c_uint32), ("n_candidates", C.c_uint32)]


class TraxConfig(C.Structure):
    _fields_ = [("n_layer_triplets", C.c_uint32),
                ("triplets", TraxLayerTriplet * MAX_LAYER_TRIPLETS),
                ("n_geom_layers", C.c_uint32),
                ("min_radius", C.c_float * MAX_LAYERS),
                ("max_radius", C.c_float * MAX_LAYERS),
                ("min_pt", C.c_float), ("bz", C.c_float)]


class TraxTuning(C.Structure):
    _fields_ = [("run_walk", C.c_uint32), ("index_min", C.c_uint32),
                ("pair_record", C.c_uint32), ("blocks_per_sm", C.c_uint32)]


class TraxHits(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("layer", C.c_void_p), ("detector_id", C.c_void_p),
                ("hit_id", C.c_void_p), ("event", C.c_void_p), ("n", C.c_uint32)]


class TraxSortedHits(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("phi", C.c_void_p),
                ("layer", C.c_void_p), ("detector_id", C.c_void_p), ("hit_id", C.c_void_p),
                ("event", C.c_void_p), ("orig", C.c_void_p), ("n", C.c_uint32)]


class TraxLayout(C.Structure):
    _fields_ = [("n_events", C.c_uint32), ("n_layers", C.c_uint32),
                ("event_nhits", C.c_void_p), ("event_offset", C.c_void_p),
                ("layer_nhits", C.c_void_p), ("layer_offset", C.c_void_p)]


class TraxPairs(C.Structure):
    _fields_ = [("pairs", C.c_void_p), ("offsets", C.c_void_p), ("capacity", C.c_uint32)]


class TraxTracklets(C.Structure):
    _fields_ = [("hit1", C.c_void_p), ("hit2", C.c_void_p), ("hit3", C.c_void_p),
                ("offsets", C.c_void_p), ("capacity", C.c_uint32)]


class TraxCounts(C.Structure):
    _fields_ = [("n_hits", C.c_uint64), ("n_pairs", C.c_uint64), ("pair_slots", C.c_uint64),
                ("n_candidates", C.c_uint64), ("cand_slots", C.c_uint64),
                ("cand_truncated", C.c_uint64), ("n_tracklets", C.c_uint64),
                ("status", C.c_uint32), ("error_detail", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class TraxEventBatch(C.Structure):
    _fields_ = [("n_events", C.c_uint32), ("n_layers", C.c_uint32), ("n_hits", C.c_uint32),
                ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("layer", C.c_void_p), ("detector_id", C.c_void_p), ("hit_id", C.c_void_p),
                ("event", C.c_void_p), ("layer_nhits", C.c_void_p)]


class TraxBatchResult(C.Structure):
    _fields_ = [("hit1", C.c_void_p), ("hit2", C.c_void_p), ("hit3", C.c_void_p),
                ("offsets", C.c_void_p), ("capacity", C.c_uint32), ("input_indices", C.c_int),
                ("n_tracklets", C.c_uint32), ("counts", TraxCounts)]


def make_config(rows, min_radius, max_radius, min_pt, bz=0.0) -> TraxConfig:
    """rows: (layer1, layer2, layer3, dThetaCut, sigmaZ, dPhiCut, sigmaPhi,
    tipCut, pairSpreadZ, z0, pairSpreadPhi, nCandidates) tuples."""
    cfg = TraxConfig()
    cfg.n_layer_triplets = len(rows)
    for i, r in enumerate(rows):
        t = cfg.triplets[i]
        (t.layer1, t.layer2, t.layer3, t.dtheta_cut, t.sigma_z, t.dphi_cut, t.sigma_phi,
         t.tip_cut, t.pair_spread_z, t.z0, t.pair_spread_phi, t.n_candidates) = (
            int(r[0]), int(r[1]), int(r[2]), float(r[3]), float(r[4]), float(r[5]),
            float(r[6]), float(r[7]), int(r[8]), float(r[9]), int(r[10]), int(r[11]))
    cfg.n_geom_layers = len(min_radius)
    for i, (a, b) in enumerate(zip(min_radius, max_radius)):
        cfg.min_radius[i] = float(a)
        cfg.max_radius[i] = float(b)
    cfg.min_pt = float(min_pt)
    cfg.bz = float(bz)
    return cfg


class TraxServerOpts(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("max_batch_events", C.c_uint32),
                ("max_event_hits", C.c_uint32), ("n_layers", C.c_uint32),
                ("n_sectors_z", C.c_uint32), ("n_sectors_phi", C.c_uint32),
                ("memory_budget_bytes", C.c_uint64), ("keep_results", C.c_int),
                ("max_batch_hits", C.c_uint32), ("pairs_per_hit", C.c_uint32),
                ("candidates_per_hit", C.c_uint32), ("tracklets_per_hit", C.c_uint32),
                ("tuning", TraxTuning)]


class TraxServerResult(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int), ("arrival_ns", C.c_uint64),
                ("start_ns", C.c_uint64), ("done_ns", C.c_uint64), ("batch_events", C.c_uint32),
                ("hit1", C.c_void_p), ("hit2", C.c_void_p), ("hit3", C.c_void_p),
                ("capacity", C.c_uint32), ("n_tracklets", C.c_uint32),
                ("offsets", C.c_uint32 * (MAX_LAYER_TRIPLETS + 1))]


class TraxServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("events", C.c_uint64), ("batches", C.c_uint64),
                ("batched_events", C.c_uint64), ("splits", C.c_uint64), ("errors", C.c_uint64),
                ("slot_max_hits", C.c_uint64), ("p50_ns", C.c_uint64), ("p99_ns", C.c_uint64),
                ("max_ns", C.c_uint64), ("sustained_events_per_s", C.c_double),
                ("slot_max_pairs", C.c_uint64), ("count_passes", C.c_uint64),
                ("deferred", C.c_uint64)]

    def as_dict(self):
        return {k: (float(getattr(self, k)) if t is C.c_double else int(getattr(self, k)))
                for k, t in self._fields_}


PB_CONTAINER, PB_EVENT_STORE = 0, 1


class TraxPbEvents(C.Structure):
    _fields_ = [("n_events", C.c_uint32), ("n_hits", C.c_uint64),
                ("run", C.c_void_p), ("lumi", C.c_void_p), ("event_number", C.c_void_p),
                ("hit_offset", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p),
                ("z", C.c_void_p), ("detector_type", C.c_void_p), ("layer", C.c_void_p),
                ("detector_id", C.c_void_p), ("hit_id", C.c_void_p),
                ("sim_track_id", C.c_void_p), ("sim_track_pt", C.c_void_p)]


class TraxRawHits(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("layer", C.c_void_p), ("detector_id", C.c_void_p),
                ("sim_track_id", C.c_void_p), ("sim_track_pt", C.c_void_p),
                ("event_offset", C.c_void_p), ("n_events", C.c_uint32), ("n_hits", C.c_uint32)]


class TraxIngestCfg(C.Structure):
    _fields_ = [("min_pt", C.c_float), ("max_layer", C.c_uint32), ("used_layers", C.c_uint32),
                ("only_tracks", C.c_int), ("num_tracks", C.c_int32)]


class TraxHitsOut(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("layer", C.c_void_p), ("detector_id", C.c_void_p), ("hit_id", C.c_void_p),
                ("event", C.c_void_p), ("capacity", C.c_uint32)]


class TraxTrackList(C.Structure):
    _fields_ = [("track_id", C.c_void_p), ("inner", C.c_void_p), ("middle", C.c_void_p),
                ("outer", C.c_void_p), ("offsets", C.c_void_p), ("capacity", C.c_uint32)]
