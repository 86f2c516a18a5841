"""Seeded synthetic barrel events for the triplet-seeding path.

The reference measures on CMS event files that are not shipped with it; these
events stand in for them with the shapes of the five benchmark workloads:
helix tracks from a beam-line vertex in a solenoid field, intersected with
concentric barrel layers, smeared, plus uniform noise hits.

Physics of one track (B along z, vertex on the beam line):
  R [cm]      = 100 * pT / (0.299792458 * B)
  phi(r)      = phi0 - q * asin(r / 2R)
  z(r)        = z_v + 2R * asin(r / 2R) * cot(theta),  cot(theta) = sinh(eta)
Each layer is a ring of staggered modules at r - 0.2 and r + 0.2 cm
(alternating in phi), so the layer's GeometrySupplement radii are r -/+ 0.25
cm.  A layer with min radius == max radius would hit the reference's
branchless max/min (PairGeneratorBeamspot.h:122,127 and
TripletThetaPhiPredictor.h:126-127 yield 0 for equal operands) and collapse
every z window to +/-sigmaZ around 0.
A hit is kept when the track reaches the module (r <= 2R) and |z| <= 26.7 cm.
pT is drawn from 1/pT^2 on [a, b] by inverse CDF, eta ~ U[-2.5, 2.5],
phi0 ~ U[-pi, pi), q = +/-1, z_v ~ N(0, 5 cm); x, y, z are smeared by
N(0, 20 um).  Noise hits: uniform in phi and z on each layer.

Hits are bucketed per event and layer, the order HitCollection::addEvent
produces (src/datastructures/HitCollection.cpp:121-146); within a layer the
order is a seeded shuffle.  `hit_id` carries the track number (0 = noise) as
the reference's HitId column carries the sim-track id (HitCollection.cpp:138).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math

import numpy as np

from ._abi import TraxConfig, TraxGridCfg, make_config

BZ_TESLA = 3.8
Z_ACCEPT_CM = 26.7
SMEAR_CM = 20e-4
SEED_BASE = 0x7A11

BARREL_RADII_CM = (4.4, 7.3, 10.2, 16.0)
MODULE_STAGGER_CM = 0.2
LAYER_HALF_THICKNESS_CM = 0.25
MODULE_WIDTH_CM = 1.6

# Layer-triplet rows of configs/layerTriplets.xml:5-35 (the reference's cut
# table): layer1..3, dThetaCut, sigmaZ, dPhiCut, sigmaPhi, tipCut,
# pairSpreadZ, z0, pairSpreadPhi, nCandidates.
LAYER_TRIPLETS_XML = (
    (1, 2, 3, 0.01, 0.037, 0.075, 0.032, 0.5, 2, 10.0, 2, 4),
    (2, 3, 4, 0.2, 0.207, 0.2, 0.102, 0.5, 2, 10.0, 2, 16),
)


@dataclass
class Workload:
    """One benchmark workload: event composition plus hot-path settings."""

    name: str
    config_id: int
    n_layers: int
    noise: float
    pt_range: tuple
    n_sectors_z: int
    n_sectors_phi: int
    n_triplets: int
    tracks: int | None = None          # fixed track count per event
    pileup_mean: float | None = None   # Poisson pile-up vertices (+1 hard vertex)
    pileup_uniform: int | None = None  # pile-up ~ U{0..n}
    tracks_per_vertex: float = 40.0
    cut_override: dict = field(default_factory=dict)
    events: int = 1

    @property
    def min_pt(self) -> float:
        return float(self.pt_range[0])

    def config(self) -> TraxConfig:
        rows = []
        for t in LAYER_TRIPLETS_XML[: self.n_triplets]:
            row = list(t)
            if "dtheta_cut" in self.cut_override:
                row[3] = self.cut_override["dtheta_cut"]
            if "dphi_cut" in self.cut_override:
                row[5] = self.cut_override["dphi_cut"]
            rows.append(tuple(row))
        radii = BARREL_RADII_CM[: self.n_layers]
        return make_config(rows, [r - LAYER_HALF_THICKNESS_CM for r in radii],
                           [r + LAYER_HALF_THICKNESS_CM for r in radii], self.min_pt)

    def grid(self, n_events: int) -> TraxGridCfg:
        return TraxGridCfg(n_events, self.n_layers, self.n_sectors_z, self.n_sectors_phi)


WORKLOADS = {
    "single-muon-100trk": Workload(
        "single-muon-100trk", 1, 3, 0.05, (1.0, 50.0), 8, 16, 1, tracks=100,
        cut_override={"dphi_cut": 0.02, "dtheta_cut": 0.01}),
    "multimuon-1000trk": Workload(
        "multimuon-1000trk", 2, 4, 0.10, (1.0, 50.0), 12, 32, 2, tracks=1000),
    "pileup50-batch100": Workload(
        "pileup50-batch100", 3, 4, 0.10, (0.9, 100.0), 12, 32, 2, pileup_mean=50.0,
        events=100),
    "pileup200": Workload(
        "pileup200", 4, 4, 0.10, (0.9, 100.0), 12, 32, 2, pileup_mean=200.0, events=64),
    "stream-pileup-u200": Workload(
        "stream-pileup-u200", 5, 4, 0.10, (0.9, 100.0), 12, 32, 2, pileup_uniform=200),
}


@dataclass
class EventBatch:
    """Host SoA hit columns of a batch of events plus its bucketing."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    layer: np.ndarray
    detector_id: np.ndarray
    hit_id: np.ndarray
    event: np.ndarray
    layer_nhits: np.ndarray  # [n_events, n_layers] uint32

    @property
    def n_events(self) -> int:
        return int(self.layer_nhits.shape[0])

    @property
    def n_layers(self) -> int:
        return int(self.layer_nhits.shape[1])

    @property
    def n_hits(self) -> int:
        return int(self.x.shape[0])

    @property
    def event_nhits(self) -> np.ndarray:
        return self.layer_nhits.sum(axis=1).astype(np.uint32)

    @property
    def event_offset(self) -> np.ndarray:
        n = self.event_nhits.astype(np.uint64)
        return (np.cumsum(n) - n).astype(np.uint32)

    @property
    def layer_offset(self) -> np.ndarray:
        """Offset of each (event, layer) bucket within its event."""
        n = self.layer_nhits.astype(np.uint64)
        return (np.cumsum(n, axis=1) - n).astype(np.uint32)

    def columns(self):
        return (self.x, self.y, self.z, self.layer, self.detector_id, self.hit_id, self.event)

    @staticmethod
    def concat(batches) -> "EventBatch":
        batches = list(batches)
        ev = []
        base = 0
        for b in batches:
            ev.append(b.event + np.uint32(base))
            base += b.n_events
        return EventBatch(
            np.concatenate([b.x for b in batches]), np.concatenate([b.y for b in batches]),
            np.concatenate([b.z for b in batches]), np.concatenate([b.layer for b in batches]),
            np.concatenate([b.detector_id for b in batches]),
            np.concatenate([b.hit_id for b in batches]), np.concatenate(ev).astype(np.uint32),
            np.concatenate([b.layer_nhits for b in batches], axis=0))

    def slice_events(self, first: int, count: int) -> "EventBatch":
        off = self.event_offset
        lo = int(off[first])
        hi = int(off[first + count - 1] + self.event_nhits[first + count - 1])
        s = slice(lo, hi)
        return EventBatch(self.x[s].copy(), self.y[s].copy(), self.z[s].copy(),
                          self.layer[s].copy(), self.detector_id[s].copy(),
                          self.hit_id[s].copy(), (self.event[s] - np.uint32(first)).astype(np.uint32),
                          self.layer_nhits[first:first + count].copy())


def generate_event(w: Workload, event_index: int, radii=None):
    """Returns per-layer lists of (x, y, z, hit_id, det_id) arrays for one event."""
    radii = BARREL_RADII_CM[: w.n_layers] if radii is None else radii
    seed = SEED_BASE + w.config_id * 1_000_000 + int(event_index)
    rng = np.random.Generator(np.random.Philox(seed))
    if w.tracks is not None:
        n_trk = int(w.tracks)
        vtx_of_track = np.zeros(n_trk, dtype=np.int64)
        vtx_z = rng.normal(0.0, 5.0, size=1)
    else:
        if w.pileup_mean is not None:
            n_vtx = 1 + int(rng.poisson(w.pileup_mean))
        else:
            n_vtx = 1 + int(rng.integers(0, int(w.pileup_uniform) + 1))
        per_vtx = rng.poisson(w.tracks_per_vertex, size=n_vtx)
        n_trk = int(per_vtx.sum())
        vtx_of_track = np.repeat(np.arange(n_vtx), per_vtx)
        vtx_z = rng.normal(0.0, 5.0, size=n_vtx)
    a, b = w.pt_range
    u = rng.random(n_trk)
    pt = 1.0 / (1.0 / a - u * (1.0 / a - 1.0 / b))
    eta = rng.uniform(-2.5, 2.5, n_trk)
    phi0 = rng.uniform(-math.pi, math.pi, n_trk)
    q = np.where(rng.random(n_trk) < 0.5, -1.0, 1.0)
    zv = vtx_z[vtx_of_track]
    R = 100.0 * pt / (0.299792458 * BZ_TESLA)
    cot = np.sinh(eta)
    layers = []
    for li, r_nom in enumerate(radii):
        n_mod = 2 * max(4, int(round(math.pi * r_nom / MODULE_WIDTH_CM)))

        def module_radius(phi):
            m = np.floor((phi + math.pi) / (2 * math.pi) * n_mod).astype(np.int64) % n_mod
            return r_nom + np.where(m % 2 == 0, -MODULE_STAGGER_CM, MODULE_STAGGER_CM)

        arg0 = np.clip(r_nom / (2.0 * R), 0.0, 1.0)
        r = module_radius(phi0 - q * np.arcsin(arg0))
        reach = r <= 2.0 * R
        arg = np.clip(r / (2.0 * R), 0.0, 1.0)
        s = 2.0 * R * np.arcsin(arg)
        phi = phi0 - q * np.arcsin(arg)
        zz = zv + s * cot
        keep = reach & (np.abs(zz) <= Z_ACCEPT_CM)
        idx = np.nonzero(keep)[0]
        xs = r[idx] * np.cos(phi[idx]) + rng.normal(0.0, SMEAR_CM, idx.size)
        ys = r[idx] * np.sin(phi[idx]) + rng.normal(0.0, SMEAR_CM, idx.size)
        zs = zz[idx] + rng.normal(0.0, SMEAR_CM, idx.size)
        hid = (idx + 1).astype(np.uint32)
        n_noise = int(round(w.noise * idx.size))
        nphi = rng.uniform(-math.pi, math.pi, n_noise)
        nr = module_radius(nphi)
        nz = rng.uniform(-Z_ACCEPT_CM, Z_ACCEPT_CM, n_noise)
        xs = np.concatenate([xs, nr * np.cos(nphi) + rng.normal(0.0, SMEAR_CM, n_noise)])
        ys = np.concatenate([ys, nr * np.sin(nphi) + rng.normal(0.0, SMEAR_CM, n_noise)])
        zs = np.concatenate([zs, nz + rng.normal(0.0, SMEAR_CM, n_noise)])
        hid = np.concatenate([hid, np.zeros(n_noise, dtype=np.uint32)])
        perm = rng.permutation(xs.size)
        xs, ys, zs, hid = xs[perm], ys[perm], zs[perm], hid[perm]
        ph = np.arctan2(ys, xs)
        det = ((li + 1) << 16) | ((np.floor((ph + math.pi) / (2 * math.pi) * n_mod).astype(np.int64) % n_mod) << 6) \
            | np.clip(np.floor((zs + Z_ACCEPT_CM) / (2 * Z_ACCEPT_CM) * 16), 0, 15).astype(np.int64)
        layers.append((xs.astype(np.float32), ys.astype(np.float32), zs.astype(np.float32),
                       hid, det.astype(np.uint32)))
    return layers


def generate_batch(w: Workload, n_events: int, first_event: int = 0) -> EventBatch:
    cols = {k: [] for k in ("x", "y", "z", "layer", "det", "hid", "event")}
    nh = np.zeros((n_events, w.n_layers), dtype=np.uint32)
    for e in range(n_events):
        layers = generate_event(w, first_event + e)
        for li, (xs, ys, zs, hid, det) in enumerate(layers):
            cols["x"].append(xs)
            cols["y"].append(ys)
            cols["z"].append(zs)
            cols["layer"].append(np.full(xs.size, li + 1, dtype=np.uint32))
            cols["det"].append(det)
            cols["hid"].append(hid)
            cols["event"].append(np.full(xs.size, e, dtype=np.uint32))
            nh[e, li] = xs.size
    cat = lambda k, dt: (np.concatenate(cols[k]).astype(dt) if cols[k] else np.zeros(0, dt))
    return EventBatch(cat("x", np.float32), cat("y", np.float32), cat("z", np.float32),
                      cat("layer", np.uint32), cat("det", np.uint32), cat("hid", np.uint32),
                      cat("event", np.uint32), nh)
