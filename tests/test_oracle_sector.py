"""The oracle's PairGeneratorSector restatement (PairGeneratorSector.h:43-230)
against the cell geometry it implements, derived independently of its loop:
an inner hit in cell (zs, ps) pairs with every layer-2 hit whose cell lies in
rows [zs - sZ, min(zs + sZ + 1, Z)) -- none when zs < sZ, where the
reference's unsigned subtraction wraps (:98) -- and in the phi columns
[ps - sP, ps + sP] taken modulo P, except that a block ending exactly on the
sentinel column P does not wrap to column 0 (the test `phiHighSector >
nSectorsPhi + 1` at :107).  Visits with repeats (pairCount's nFound) are the
pair slots."""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg


def cell_of(seg_grid, idx):
    return np.searchsorted(seg_grid, idx, side="right") - 1


def columns(ps, s, P):
    lo, hi = ps - s, ps + s + 1
    wrap = lo < 0 or hi > P + 1
    if lo < 0:
        lo += P
    if hi > P + 1:
        hi -= P
    if wrap:
        return list(range(lo, P)) + list(range(0, hi))  # with repeats
    return list(range(lo, min(hi, P)))


def expected(res, cfg, grid):
    E, L, Z, P = grid.n_events, grid.n_layers, grid.n_sectors_z, grid.n_sectors_phi
    C = (Z + 1) * (P + 1)
    g = res["grid"].reshape(E, L, C)
    pairs, offsets, slots = [], [0], 0
    for e in range(E):
        for t in range(cfg.n_layer_triplets):
            lt = cfg.triplets[t]
            g1, g2 = g[e, lt.layer1 - 1], g[e, lt.layer2 - 1]
            sZ, sP = lt.pair_spread_z, lt.pair_spread_phi
            outer = np.arange(g2[0], g2[C - 1])
            oc = cell_of(g2, outer)
            ozs, ops = oc // (P + 1), oc % (P + 1)
            assert (ops < P).all()  # no hit sits at phi = +pi exactly
            count = np.zeros((Z + 1, P + 1), np.int64)
            np.add.at(count, (ozs, ops), 1)
            for h in range(g1[0], g1[C - 1]):
                c = cell_of(g1, h)
                zs, ps = c // (P + 1), c % (P + 1)
                rows = range(zs - sZ, min(zs + sZ + 1, Z)) if zs >= sZ else range(0)
                cols = columns(ps, sP, P)
                slots += sum(int(count[r, q]) for r in rows for q in cols)
                sel = np.isin(ozs, list(rows)) & np.isin(ops, cols)
                pairs.extend((h, int(o)) for o in outer[sel])
            offsets.append(len(pairs))
    return np.array(pairs, np.uint32).reshape(-1, 2), np.array(offsets, np.uint32), slots


CASES = [("single-muon-100trk", 3, None), ("multimuon-1000trk", 1, None),
         ("multimuon-1000trk", 2, (4, 4)), ("multimuon-1000trk", 1, (3, 3)),
         ("pileup50-batch100", 1, (64, 128))]


@pytest.mark.parametrize("name,n_ev,zp", CASES)
def test_sector_pairs_follow_cell_geometry(name, n_ev, zp):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    cfg = w.config()
    grid = w.grid(n_ev) if zp is None else TraxGridCfg(n_ev, w.n_layers, *zp)
    r = oracle.run(b, cfg, grid, 2, n_threads=1, pair_gen="sector")
    assert r["stats"]["status"] == 0
    want, want_off, want_slots = expected(r, cfg, grid)
    got = oracle.canonical(r)["pairs"]
    assert np.array_equal(got, want)
    assert r["stats"]["pair_slots"] == want_slots
    if want_slots == len(want):
        assert np.array_equal(r["pair_offsets"], want_off)
    else:  # repeated visits leave unwritten slots at each group's end
        assert r["stats"]["pairs"] == len(want) < want_slots


def test_small_grid_has_repeats_and_z_underflow():
    """On a 4 x 4 grid a spread of 2 covers more than the row, so cells are
    visited twice, and hits in z sector 1 (< pairSpreadZ) find nothing."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 1)
    grid = TraxGridCfg(1, w.n_layers, 4, 4)
    r = oracle.run(b, w.config(), grid, 2, n_threads=1, pair_gen="sector")
    st = r["stats"]
    assert st["pair_slots"] > st["pairs"] > 0
    C = 5 * 5
    g1 = r["grid"][:C]  # event 0, layer 1
    in_z1 = np.arange(g1[1 * 5], g1[2 * 5])
    assert in_z1.size > 0
    assert not np.isin(oracle.canonical(r)["pairs"][:, 0], in_z1).any()


@pytest.mark.parametrize("n_threads", [1, 64, 256])  # power-of-two work groups, as PrefixSum needs
def test_sector_thread_layouts_agree(n_threads):
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 2)
    base = oracle.run(b, w.config(), w.grid(2), 4, n_threads=1, pair_gen="sector")
    r = oracle.run(b, w.config(), w.grid(2), 4, n_threads=n_threads, pair_gen="sector")
    as_set = lambda a: set(map(tuple, np.asarray(a).tolist()))
    cb, cr = oracle.canonical(base), oracle.canonical(r)
    assert as_set(cb["pairs"]) == as_set(cr["pairs"])
    assert np.array_equal(base["pair_offsets"], r["pair_offsets"])
    assert r["stats"]["tracklets"] > 0
