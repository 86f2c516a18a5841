"""CPU tests of the oracle: the reference's own self-checks, hand-derived
known answers, and consistency of the restatement."""
import math

import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg, make_config

# ---------------------------------------------------------------------------
# Project FP32 math against float64 libm.


def _ulp_err(got, ref):
    ref32 = np.abs(ref).astype(np.float32)
    ulp = np.spacing(np.maximum(ref32, np.float32(1e-30))).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref) / ulp


def test_atan2_accuracy():
    rng = np.random.default_rng(1)
    y = rng.normal(0, 10, 200_000).astype(np.float32)
    x = rng.normal(0, 10, 200_000).astype(np.float32)
    got = oracle.math_batch(0, y, x)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert _ulp_err(got, ref).max() <= 4.0
    assert np.all(np.abs(got) <= np.float32(math.pi) + 0)  # within [-pi_f, pi_f]


def test_atan2_special_values():
    pi_f = np.float32(math.pi)
    cases = [(0.0, 1.0, 0.0), (0.0, -1.0, pi_f), (-0.0, -1.0, -pi_f), (1.0, 0.0, pi_f / 2),
             (-1.0, 0.0, -pi_f / 2), (0.0, 0.0, 0.0), (0.0, -0.0, pi_f)]
    for yy, xx, want in cases:
        got = oracle.math_batch(0, np.array([yy], np.float32), np.array([xx], np.float32))[0]
        assert got == np.float32(want), (yy, xx, got, want)
    assert np.isnan(oracle.math_batch(0, np.array([np.nan], np.float32), np.array([1.0], np.float32))[0])


def test_acos_atan_accuracy():
    rng = np.random.default_rng(2)
    a = rng.uniform(-1, 1, 200_000).astype(np.float32)
    got = oracle.math_batch(1, a)
    ref = np.arccos(a.astype(np.float64))
    assert _ulp_err(got, ref).max() <= 8.0
    t = rng.normal(0, 5, 200_000).astype(np.float32)
    got = oracle.math_batch(2, t)
    assert _ulp_err(got, np.arctan(t.astype(np.float64))).max() <= 4.0
    assert np.isnan(oracle.math_batch(1, np.array([1.5], np.float32))[0])
    assert oracle.math_batch(1, np.array([1.0], np.float32))[0] == 0.0
    assert oracle.math_batch(1, np.array([-1.0], np.float32))[0] == np.float32(math.pi)


def test_min_radius_curvature():
    # TripletConfiguration.cpp:145-152 at 1 GeV and IDEAL_BZ = 3.8112
    r = oracle.lib().or_min_radius_curvature(1.0, 0.0)
    want = np.float32(1.0 * 5.344286e-19 / (np.float64(np.float32(3.8112)) * 1.602177e-19) * 100.0)
    assert np.float32(r) == want
    assert abs(r - 87.522) < 1e-2


# ---------------------------------------------------------------------------
# PrefixSum: the reference's own self-check (trax_test.cpp:473-479) and
# agreement with a plain exclusive scan for every work-group size.


@pytest.mark.parametrize("wg", [128, 256])
def test_prefix_sum_all_ones_1mi(wg):
    n = 1024 * 1024
    out = oracle.prefix_sum(np.ones(n, np.uint32), wg)
    assert out[n - 1] == n - 1
    assert np.array_equal(out, np.arange(n, dtype=np.uint32))


@pytest.mark.parametrize("wg", [1, 2, 4, 16, 64, 256, 512])
@pytest.mark.parametrize("n", [1, 2, 3, 31, 1000, 4097])
def test_prefix_sum_matches_exclusive_scan(wg, n):
    v = np.random.default_rng(n * 7 + wg).integers(0, 50, n).astype(np.uint32)
    out = oracle.prefix_sum(v, wg)
    ref = np.concatenate([[0], np.cumsum(v)[:-1]]).astype(np.uint32)
    assert np.array_equal(out, ref)


# ---------------------------------------------------------------------------
# Grid invariants: GridBuilder::verifyGrid (GridBuilder.cpp:187-224).


def verify_grid(res, n_events, n_layers, nz, nphi):
    C = (nz + 1) * (nphi + 1)
    grid = res["grid"].reshape(n_events, n_layers, nz + 1, nphi + 1)
    szz = np.float32(600.0) / np.float32(nz)
    szp = np.float32(2 * np.float32(math.pi)) / np.float32(nphi)
    z = res["sorted_z"]
    phi = res["sorted_phi"]
    flat = res["grid"]
    assert np.all(np.diff(flat.astype(np.int64)) >= 0), "grid not monotone"
    for e in range(n_events):
        for l in range(n_layers):
            g = grid[e, l]
            for zi in range(nz):
                for p in range(nphi):
                    lo, hi = g[zi, p], g[zi, p + 1]
                    if hi <= lo:
                        continue
                    assert np.all(res["sorted_layer"][lo:hi] == l + 1)
                    assert np.all(res["sorted_event"][lo:hi] == e)
                    zb0 = np.float32(-300) + np.float32(zi) * szz
                    zb1 = np.float32(-300) + np.float32(zi + 1) * szz
                    assert np.all((z[lo:hi] >= zb0) & (z[lo:hi] <= zb1))
                    pb0 = np.float32(-math.pi) + np.float32(p) * szp
                    pb1 = np.float32(-math.pi) + np.float32(p + 1) * szp
                    assert np.all((phi[lo:hi] >= pb0 - 1e-6) & (phi[lo:hi] <= pb1 + 1e-6))
    assert np.array_equal(np.sort(res["sorted_orig"]), np.arange(z.size, dtype=np.uint32))


@pytest.mark.parametrize("name,n_ev", [("single-muon-100trk", 2), ("multimuon-1000trk", 2),
                                       ("pileup50-batch100", 2)])
def test_grid_invariants(name, n_ev):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    r = oracle.run(b, w.config(), w.grid(n_ev), n_stages=1, n_threads=256)
    assert r["stats"]["status"] == 0
    verify_grid(r, n_ev, w.n_layers, w.n_sectors_z, w.n_sectors_phi)
    # stable: input order kept within a cell
    orig = r["sorted_orig"]
    grid = r["grid"]
    for s in range(0, grid.size - 1):
        lo, hi = grid[s], grid[s + 1]
        if hi - lo > 1:
            assert np.all(np.diff(orig[lo:hi].astype(np.int64)) > 0)
    # the sorted columns are a permutation of the input
    assert np.array_equal(r["sorted_x"], b.x[orig])
    assert np.array_equal(r["sorted_hitid"], b.hit_id[orig])


# ---------------------------------------------------------------------------
# Consistency: thread layouts and OpenMP give the same sets.


def _sets(res):
    c = oracle.canonical(res)
    return {k: set(map(tuple, v.tolist())) for k, v in c.items()}


@pytest.mark.parametrize("name,n_ev", [("multimuon-1000trk", 2), ("pileup50-batch100", 2)])
def test_thread_layout_and_omp_agree(name, n_ev):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    cfg, g = w.config(), w.grid(n_ev)
    r1 = oracle.run(b, cfg, g, 4, 1, 1)
    r256 = oracle.run(b, cfg, g, 4, 256, 1)
    romp = oracle.run(b, cfg, g, 4, 256, 4)
    assert _sets(r1) == _sets(r256)
    for k in ("grid", "pairs", "pair_offsets", "cands", "cand_offsets", "trk_h1", "trk_offsets"):
        assert np.array_equal(r256[k], romp[k]), k
    assert r1["pair_offsets"].tolist() == r256["pair_offsets"].tolist()
    assert r1["trk_offsets"].tolist() == r256["trk_offsets"].tolist()
    s = r1["stats"]
    assert s["status"] == 0
    assert s["pairs"] == s["pair_slots"]  # no unwritten pair slots on these configs
    assert s["tracklets"] > 0


# ---------------------------------------------------------------------------
# Hand-derived known answers.

RADII = (4.4, 7.3, 10.2)


def _helix_hits(pt, eta, phi0, q, zv, radii=RADII, bz=3.8):
    R = 100.0 * pt / (0.299792458 * bz)
    out = []
    for r in radii:
        a = r / (2 * R)
        phi = phi0 - q * math.asin(a)
        s = 2 * R * math.asin(a)
        out.append((r * math.cos(phi), r * math.sin(phi), zv + s * math.sinh(eta)))
    return out


def _batch(tracks, noise=()):
    """tracks: lists of per-layer (x, y, z); builds one bucketed event."""
    layers = [[] for _ in RADII]
    for tid, hits in enumerate(tracks, start=1):
        for li, h in enumerate(hits):
            layers[li].append((h, tid))
    for li, h in noise:
        layers[li].append((h, 0))
    xs, ys, zs, ly, hid = [], [], [], [], []
    for li, hs in enumerate(layers):
        for (x, y, z), t in hs:
            xs.append(x); ys.append(y); zs.append(z); ly.append(li + 1); hid.append(t)
    n = len(xs)
    return gen.EventBatch(np.array(xs, np.float32), np.array(ys, np.float32),
                          np.array(zs, np.float32), np.array(ly, np.uint32),
                          np.zeros(n, np.uint32), np.array(hid, np.uint32),
                          np.zeros(n, np.uint32),
                          np.array([[len(h) for h in layers]], np.uint32))


def _cfg(min_r=(4.15, 7.05, 9.95), max_r=(4.65, 7.55, 10.45)):
    row = (1, 2, 3, 0.01, 0.037, 0.02, 0.032, 0.5, 2, 10.0, 2, 4)
    return make_config([row], min_r, max_r, 1.0)


def test_known_answer_single_track():
    """A 5 GeV track from z=1 cm: its three hits form the only pair, the only
    candidate and the only tracklet (windows contain the true hits since
    pT > minPt and |z_v| < z0; the triplet is straight in r-z, bends by
    ~2e-3 rad in phi and points at the beam line)."""
    b = _batch([_helix_hits(5.0, 0.3, 0.5, +1, 1.0)])
    r = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 4, 256)
    c = oracle.canonical(r)
    assert c["pairs"].tolist() == [[0, 1]]
    assert c["cand_hits"].tolist() == [[0, 1, 2]]
    assert c["tracklets"].tolist() == [[0, 1, 2]]
    assert r["trk_offsets"].tolist() == [0, 1]
    assert r["pair_offsets"].tolist() == [0, 1]


def test_known_answer_low_pt_rejected_and_combinatorics():
    """Two 5 GeV tracks 1 rad apart give exactly their own two tracklets; a
    0.4 GeV track (radius 35 cm < minRadius 87.5 cm) gives none."""
    t1 = _helix_hits(5.0, 0.3, 0.5, +1, 1.0)
    t2 = _helix_hits(5.0, -0.4, 1.5, -1, -2.0)
    t3 = _helix_hits(0.4, 0.1, -2.0, +1, 0.5)
    b = _batch([t1, t2, t3])
    r = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 4, 256)
    trk = oracle.canonical(r)["tracklets"]
    hid = b.hit_id[r["sorted_orig"]]
    ids = sorted({tuple(hid[list(t)]) for t in trk.tolist()})
    assert ids == [(1, 1, 1), (2, 2, 2)]


def test_known_answer_phi_wraparound():
    """A track crossing phi = +-pi is still found: the phi window wraps
    (PairGeneratorBeamspot.h:152-162, TripletThetaPhiPredictor.h:157-166)."""
    t = _helix_hits(3.0, 0.2, math.pi - 0.012, -1, 0.0)
    phis = [math.atan2(y, x) for x, y, _ in t]
    assert phis[0] > 0 and phis[2] < 0  # crosses the seam
    b = _batch([t])
    r = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 4, 256)
    assert oracle.canonical(r)["tracklets"].tolist() == [[0, 1, 2]]


def test_equal_radii_collapse_z_window():
    """min radius == max radius hits the branchless max/min of
    PairGeneratorBeamspot.h:122,127 (equal operands give 0): the z window
    shrinks to +-sigmaZ around 0, so a track at z ~ 5 cm forms no pair."""
    t = _helix_hits(5.0, 0.8, 0.5, +1, 2.0)
    b = _batch([t])
    r = oracle.run(b, _cfg(RADII, RADII), TraxGridCfg(1, 3, 8, 16), 2, 256)
    assert r["stats"]["pairs"] == 0
    r2 = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 2, 256)
    assert r2["stats"]["pairs"] == 1


def test_out_of_grid_hit_flagged():
    t = _helix_hits(5.0, 0.3, 0.5, +1, 1.0)
    t[1] = (t[1][0], t[1][1], 400.0)  # |z| > 300 cm
    b = _batch([t])
    r = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 1, 256)
    assert r["stats"]["status"] == 6 and r["stats"]["detail"] == 1


def test_empty_event_and_empty_layers():
    b = _batch([])
    r = oracle.run(b, _cfg(), TraxGridCfg(1, 3, 8, 16), 4, 256)
    assert r["stats"]["tracklets"] == 0 and r["stats"]["pairs"] == 0
    assert r["trk_offsets"].tolist() == [0, 0]


def test_float_to_int_casts_match_their_definition():
    """trax_f2u / trax_f2i (the reference's implicit casts of floor results):
    low 32 bits of the 64-bit truncation, 0 for NaN and beyond +-2^63;
    int32 truncation, INT_MIN for NaN and out of range."""
    rng = np.random.default_rng(3)
    v = np.concatenate([rng.normal(0, 10, 20000), rng.normal(0, 1e9, 20000),
                        10.0 ** rng.uniform(0, 19, 20000) * rng.choice([-1, 1], 20000),
                        [0.0, -0.0, 0.5, -0.5, -1.0, 2.0**31, -2.0**31, 2.0**32, 2.0**63,
                         -2.0**63, np.inf, -np.inf, np.nan, 1e-40]]).astype(np.float32)
    u = oracle.math_batch(3, v).view(np.uint32)
    i = oracle.math_batch(4, v).view(np.int32)
    lim = np.float32(9.2233715e18)
    for x, gu, gi in zip(v.tolist(), u.tolist(), i.tolist()):
        if x != x or abs(x) >= lim:
            assert gu == 0
        else:
            assert gu == (int(np.trunc(x)) & 0xFFFFFFFF), x
        if x != x or x >= 2.0**31 or x < -2.0**31:
            assert gi == -2**31
        else:
            assert gi == int(np.trunc(x)), x


def floor_div_cases(seed=9):
    """Numerators around every sector boundary of every grid size the
    autotuner and the configs use, plus random ones."""
    rng = np.random.default_rng(seed)
    xs, ds = [], []
    for n in list(range(1, 130)) + [256, 512]:
        for extent in (np.float32(600.0), np.float32(2 * np.float32(np.pi))):
            d = np.float32(extent / np.float32(n))
            k = np.arange(-2, n + 3, dtype=np.float32)
            base = (k * d).astype(np.float32)
            for ulps in range(-4, 5):
                xs.append(np.nextafter(base, np.float32(np.inf) if ulps > 0 else np.float32(-np.inf))
                          if ulps else base)
                for _ in range(abs(ulps) - 1):
                    xs[-1] = np.nextafter(xs[-1], np.float32(np.inf) if ulps > 0 else np.float32(-np.inf))
                ds.append(np.full(len(k), d, np.float32))
            xs.append(rng.uniform(-50, float(extent) + 50, 4000).astype(np.float32))
            ds.append(np.full(4000, d, np.float32))
    x = np.concatenate(xs + [np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 3e38, 1e-40],
                                      np.float32)])
    d = np.concatenate(ds + [np.full(7, np.float32(50.0), np.float32)])
    return x.astype(np.float32), d.astype(np.float32)


def test_reciprocal_floor_div_equals_division():
    """trax_floor_div (the kernels' sector floors through 1/d) gives
    floorf(x / d) bit for bit, including next to every cell boundary."""
    x, d = floor_div_cases()
    assert oracle.lib().or_floor_div_mismatches(oracle._ptr(x), oracle._ptr(d), x.size) == 0
