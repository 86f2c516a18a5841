"""The oracle reproduces the committed golden vectors (on any machine)."""
import numpy as np
import pytest

import oracle
from golden_util import fixtures, load


@pytest.mark.parametrize("path", fixtures())
def test_oracle_reproduces_golden(path):
    b, cfg, grid, d = load(path)
    r = oracle.run(b, cfg, grid, 4, n_threads=1)
    c = oracle.canonical(r)
    assert np.array_equal(r["grid"], d["out_grid"])
    assert np.array_equal(r["sorted_orig"], d["out_orig"])
    assert np.array_equal(c["pairs"], d["out_pairs"])
    assert np.array_equal(r["pair_offsets"], d["out_pair_offsets"])
    assert np.array_equal(c["cand_hits"], d["out_cand_hits"])
    assert np.array_equal(c["tracklets"], d["out_tracklets"])
    assert np.array_equal(r["trk_offsets"], d["out_trk_offsets"])
    st = r["stats"]
    assert [st[k] for k in ("pair_slots", "pairs", "cand_slots", "cands", "cand_truncated",
                            "tracklets")] == d["stats"].tolist()


def test_fixtures_present():
    assert len(fixtures()) >= 3
