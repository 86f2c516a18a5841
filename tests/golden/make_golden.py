"""Writes the golden fixtures: seeded synthetic inputs and the oracle's
outputs for them (grid, sorted order, pairs, candidates as hit triples,
tracklets, offsets, slot counts).

    python tests/golden/make_golden.py

The oracle is the CPU restatement in oracle/; these files pin it against
itself across machines and pin the GPU path against stored vectors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from trax_gb300 import gen  # noqa: E402

CASES = (("single-muon-100trk", 3), ("multimuon-1000trk", 1), ("pileup50-batch100", 1))


def config_rows(cfg):
    rows = []
    for i in range(cfg.n_layer_triplets):
        t = cfg.triplets[i]
        rows.append((t.layer1, t.layer2, t.layer3, t.dtheta_cut, t.sigma_z, t.dphi_cut,
                     t.sigma_phi, t.tip_cut, t.pair_spread_z, t.z0, t.pair_spread_phi,
                     t.n_candidates))
    return np.array(rows, dtype=np.float64)


def main():
    for name, n_ev in CASES:
        w = gen.WORKLOADS[name]
        b = gen.generate_batch(w, n_ev)
        cfg, g = w.config(), w.grid(n_ev)
        r = oracle.run(b, cfg, g, 4, n_threads=1)
        c = oracle.canonical(r)
        st = r["stats"]
        np.savez_compressed(
            os.path.join(HERE, f"{name}_{n_ev}ev.npz"),
            x=b.x, y=b.y, z=b.z, layer=b.layer, detector_id=b.detector_id, hit_id=b.hit_id,
            event=b.event, layer_nhits=b.layer_nhits,
            lt_rows=config_rows(cfg),
            min_radius=np.array(cfg.min_radius[: cfg.n_geom_layers], np.float32),
            max_radius=np.array(cfg.max_radius[: cfg.n_geom_layers], np.float32),
            min_pt=np.float32(cfg.min_pt), grid=np.array([g.n_events, g.n_layers,
                                                          g.n_sectors_z, g.n_sectors_phi]),
            out_grid=r["grid"], out_orig=r["sorted_orig"], out_pairs=c["pairs"],
            out_pair_offsets=r["pair_offsets"], out_cand_hits=c["cand_hits"],
            out_tracklets=c["tracklets"], out_trk_offsets=r["trk_offsets"],
            stats=np.array([st["pair_slots"], st["pairs"], st["cand_slots"], st["cands"],
                            st["cand_truncated"], st["tracklets"]], np.uint64))
        print(name, n_ev, "hits", b.n_hits, "tracklets", st["tracklets"])


if __name__ == "__main__":
    main()
