"""The C++ operator chain (include/trax_ops.hpp, tests/cpp/ops_chain.cpp)
on the GPU equals the committed golden vectors, and its TripletConnectivity
equals the oracle's."""
import numpy as np
import pytest

import oracle
from cpp_chain import compile_chain, run_chain
from golden_util import fixtures, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chain(tmp_path_factory):
    return compile_chain(str(tmp_path_factory.mktemp("cpp")))


@pytest.mark.parametrize("path", fixtures())
def test_cpp_chain_matches_golden(gpu_ctx, chain, tmp_path, path):
    b, cfg, grid, d = load(path)
    p, out = run_chain(chain, b, cfg, grid, str(tmp_path))
    assert p.returncode == 0, p.stderr
    assert np.array_equal(out["grid"], d["out_grid"])
    assert np.array_equal(out["orig"], d["out_orig"])
    assert np.array_equal(out["pairs"], d["out_pairs"])
    assert np.array_equal(out["pair_offsets"], d["out_pair_offsets"])
    pr, c = out["pairs"], out["cands"]
    ch = np.stack([pr[c[:, 0], 0], pr[c[:, 0], 1], c[:, 1]], axis=1) if len(c) else c.reshape(0, 3)
    assert np.array_equal(ch, d["out_cand_hits"].reshape(-1, 3))
    trk = np.stack([out["hit1"], out["hit2"], out["hit3"]], axis=1)
    assert np.array_equal(trk, d["out_tracklets"].reshape(-1, 3))
    assert np.array_equal(out["trk_offsets"], d["out_trk_offsets"])
    zeros = np.zeros(len(trk), np.uint32)
    assert np.array_equal(out["connectivity"], oracle.connectivity(trk, zeros, trk, zeros))
