"""Writes the golden fixtures: seeded synthetic inputs and the reference's
outputs for them (grid, sorted order, pairs, candidates as hit triples,
tracklets, offsets, slot counts).

    python tests/golden/make_golden.py

The outputs come from the reference's own OpenCL kernels, compiled for the
host by oracle/ref_build.py (it needs the reference tree, so this script runs
where the tree is), with one work-item per grid work-group so that the
within-cell order is the input order.  The input position of each sorted hit
is read back through the DetectorId column, which the seeding kernels only
copy: the run gives each hit its own position there.  The one figure the
reference's chain does not produce -- how many store-window accepts the
prediction store drops at the count -- comes from the CPU restatement in
oracle/, after checking that the restatement reproduces every other output.
These files pin the restatement on any machine (tests/test_golden.py) and the
GPU path against stored vectors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref  # noqa: E402
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
        tagged = gen.EventBatch(b.x, b.y, b.z, b.layer, np.arange(b.n_hits, dtype=np.uint32),
                                b.hit_id, b.event, b.layer_nhits)
        r = ref.run(tagged, cfg, g, 4, n_threads=1, grid_threads=1)
        assert r["stats"]["status"] == 0, r["stats"]
        r["sorted_orig"] = r["sorted_det"]
        o = oracle.run(b, cfg, g, 4, n_threads=1)
        for k in ("grid", "sorted_orig", "pair_offsets", "cand_offsets", "trk_h1", "trk_h2",
                  "trk_h3", "trk_offsets"):
            assert np.array_equal(o[k], r[k]), k
        c = oracle.canonical(r)
        st = dict(r["stats"], cand_truncated=o["stats"]["cand_truncated"])
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
