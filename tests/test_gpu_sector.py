"""GPU parity of the sector pair generator (PairGeneratorSector) and of the
whole chain run on its pairs, against the oracle: bit-exact pairs (distinct,
in the reference's bitmap order), pair slots, offsets and tracklets."""
import numpy as np
import pytest

import oracle
from cpp_chain import compile_chain, run_chain
from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg
from trax_gb300.ops import Pipeline, build_triplets

pytestmark = pytest.mark.gpu

CASES = [("single-muon-100trk", 3, None), ("multimuon-1000trk", 1, None),
         ("multimuon-1000trk", 2, (4, 4)), ("multimuon-1000trk", 1, (3, 3)),
         ("pileup50-batch100", 2, None), ("pileup50-batch100", 1, (64, 128))]


def grid_for(w, n_ev, zp):
    return w.grid(n_ev) if zp is None else TraxGridCfg(n_ev, w.n_layers, *zp)


@pytest.mark.parametrize("name,n_ev,zp", CASES)
def test_sector_chain_bit_exact(gpu_ctx, name, n_ev, zp):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    cfg, grid = w.config(), grid_for(w, n_ev, zp)
    r = oracle.run(b, cfg, grid, 4, n_threads=1, pair_gen="sector")
    assert r["stats"]["status"] == 0
    oc = oracle.canonical(r)
    hits, g, pairs, cands, trk = build_triplets(gpu_ctx, b, cfg, grid.n_sectors_z,
                                                grid.n_sectors_phi, pair_generator="sector")
    st = r["stats"]
    p = pairs.get_pairings()
    assert np.array_equal(p, oc["pairs"])
    assert pairs.count == st["pairs"]
    if st["pairs"] == st["pair_slots"]:
        assert np.array_equal(pairs.get_pairing_offsets(), r["pair_offsets"])
    c = cands.get_pairings()
    ch = np.stack([p[c[:, 0], 0], p[c[:, 0], 1], c[:, 1]], axis=1) if len(c) else c.reshape(0, 3)
    assert np.array_equal(ch, oc["cand_hits"])
    assert np.array_equal(trk.hits(), oc["tracklets"])
    assert np.array_equal(trk.get_tracklet_offsets(), r["trk_offsets"])


def test_sector_pair_slots_counted(gpu_ctx):
    """On a 4 x 4 grid cells are visited twice: the device's slot total is
    the reference's pairCount total, the pairs are the distinct ones."""
    from trax_gb300.ops import GridBuilder, Grid, HitCollection, PairGeneratorSector, supplements
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 2)
    cfg = w.config()
    grid = TraxGridCfg(2, w.n_layers, 4, 4)
    r = oracle.run(b, cfg, grid, 2, n_threads=1, pair_gen="sector")
    gpu_ctx.configure(cfg)
    hits = HitCollection(gpu_ctx, b)
    es, ls = supplements(b)
    g = Grid(gpu_ctx, 2, w.n_layers, 4, 4)
    GridBuilder(gpu_ctx).run(hits, 256, es, ls, g)
    op = PairGeneratorSector(gpu_ctx)
    pairs = op.run(hits, cfg, 256, cfg, g)
    assert op.counts["pair_slots"] == r["stats"]["pair_slots"] > pairs.count
    assert pairs.count == r["stats"]["pairs"]


def test_sector_sets_equal_reference_thread_layout(gpu_ctx):
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 2)
    r = oracle.run(b, w.config(), w.grid(2), 4, n_threads=256, pair_gen="sector")
    oc = oracle.canonical(r)
    _, _, pairs, _, trk = build_triplets(gpu_ctx, b, w.config(), w.n_sectors_z, w.n_sectors_phi,
                                         pair_generator="sector")
    as_set = lambda a: set(map(tuple, np.asarray(a).tolist()))
    assert as_set(pairs.get_pairings()) == as_set(oc["pairs"])
    assert as_set(trk.hits()) == as_set(oc["tracklets"])


def test_sector_pipeline_and_switch_back(gpu_ctx):
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 3)
    cfg = w.config()
    want = {}
    for gen_name in ("sector", "beamspot"):
        want[gen_name] = oracle.canonical(oracle.run(b, cfg, w.grid(3), 4, n_threads=1,
                                                     pair_gen=gen_name))["tracklets"]
    p = Pipeline(gpu_ctx, cfg, w.grid(3), 3, b.n_hits, 400 * b.n_hits, 400 * b.n_hits,
                 4 * b.n_hits, pair_generator="sector")
    try:
        for _ in range(2):
            trk, _, counts = p.seed(b)
            assert counts["status"] == 0
            assert np.array_equal(trk, want["sector"])
        gpu_ctx.set_pair_generator("beamspot")
        trk, _, counts = p.seed(b)
        assert counts["status"] == 0
        assert np.array_equal(trk, want["beamspot"])
    finally:
        gpu_ctx.set_pair_generator("beamspot")


def test_cpp_sector_chain(gpu_ctx, tmp_path):
    exe = compile_chain(str(tmp_path))
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 2)
    cfg, grid = w.config(), w.grid(2)
    r = oracle.run(b, cfg, grid, 4, n_threads=1, pair_gen="sector")
    oc = oracle.canonical(r)
    proc, out = run_chain(exe, b, cfg, grid, str(tmp_path), "sector")
    assert proc.returncode == 0, proc.stderr
    assert np.array_equal(out["pairs"], oc["pairs"])
    trk = np.stack([out["hit1"], out["hit2"], out["hit3"]], axis=1)
    assert np.array_equal(trk, oc["tracklets"])
    assert np.array_equal(out["trk_offsets"], r["trk_offsets"])
