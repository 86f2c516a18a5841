"""Loads the golden fixtures of tests/golden/ (written by make_golden.py)."""
import glob
import os

import numpy as np

from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg, make_config

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixtures():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(path):
    d = np.load(path)
    b = gen.EventBatch(d["x"], d["y"], d["z"], d["layer"], d["detector_id"], d["hit_id"],
                       d["event"], d["layer_nhits"])
    rows = [tuple(r) for r in d["lt_rows"]]
    cfg = make_config(rows, d["min_radius"].tolist(), d["max_radius"].tolist(),
                      float(d["min_pt"]))
    g = d["grid"]
    grid = TraxGridCfg(int(g[0]), int(g[1]), int(g[2]), int(g[3]))
    return b, cfg, grid, d
