"""The GPU path through the C-ABI equals the committed golden vectors."""
import numpy as np
import pytest

from golden_util import fixtures, load
from trax_gb300.ops import build_triplets

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", fixtures())
def test_gpu_matches_golden(gpu_ctx, path):
    b, cfg, grid, d = load(path)
    hits, g, pairs, cands, trk = build_triplets(gpu_ctx, b, cfg, grid.n_sectors_z,
                                                grid.n_sectors_phi)
    assert np.array_equal(g.download(), d["out_grid"])
    assert np.array_equal(hits.download()["orig"], d["out_orig"])
    p = pairs.get_pairings()
    assert np.array_equal(p, d["out_pairs"])
    assert np.array_equal(pairs.get_pairing_offsets(), d["out_pair_offsets"])
    c = cands.get_pairings()
    ch = np.stack([p[c[:, 0], 0], p[c[:, 0], 1], c[:, 1]], axis=1) if len(c) else c
    assert np.array_equal(ch, d["out_cand_hits"])
    assert np.array_equal(trk.hits(), d["out_tracklets"])
    assert np.array_equal(trk.get_tracklet_offsets(), d["out_trk_offsets"])
