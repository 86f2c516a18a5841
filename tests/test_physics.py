"""Physics evaluation on the CPU: the project's FP64 asinh, the host-side
PhysicsRecords aggregation (merge arithmetic, CSV text) on a hand-computed
case, and the whole chain on the reference's ttbar events through the
oracle (a loose realism check: the data behind the reference's published
physics table is not shipped)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from trax_gb300 import gen, ingest
from trax_gb300._abi import make_config

from oracle.ref_build import DEFAULT_REFERENCE as REF  # noqa: E402

TTBAR = os.path.join(REF, "plotting", "data", "physics", "hits.ttBar.pb")


@pytest.fixture(scope="module")
def lib():
    from trax_gb300 import build, load_library
    build.build()
    return load_library()


def test_project_asinh_within_3_ulp():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 120
    rng = np.random.default_rng(1)
    ts = np.concatenate([rng.normal(0, 3, 4000), rng.uniform(-1e-6, 1e-6, 500),
                         10 ** rng.uniform(-20, 300, 500) * rng.choice([-1, 1], 500),
                         [1e-300, 5e-324, 2.0, 2.0000000001, 1.999999999]])
    for t in ts:
        a = oracle.lib().or_asinh(float(t))
        r = float(mpmath.asinh(mpmath.mpf(float(t))))
        assert abs(a - r) <= 3 * np.spacing(abs(r)), t
    assert oracle.lib().or_asinh(-0.0) == 0.0 and np.isnan(oracle.lib().or_asinh(float("nan")))


class Rec:
    def __init__(self, lib):
        self.lib = lib
        self.h = C.c_void_p()
        assert lib.trax_physics_create(C.byref(self.h)) == 0

    def add(self, e, lt, counts, cat, eta, pt, meta, mpt):
        c = np.array(counts, np.uint32)
        cat, eta, pt = (np.array(cat, np.uint8), np.array(eta, np.float64),
                        np.array(pt, np.float64))
        meta, mpt = np.array(meta, np.float64), np.array(mpt, np.float64)
        p = lambda a: a.ctypes.data if a.size else None
        assert self.lib.trax_physics_add_group(self.h, e, lt, c.ctypes.data, p(cat), p(eta), p(pt),
                                               len(cat), p(meta), p(mpt), len(meta)) == 0

    def text(self, what=0, lt=0):
        n = C.c_size_t(0)
        assert self.lib.trax_physics_csv(self.h, what, lt, None, 0, C.byref(n)) == 0
        buf = C.create_string_buffer(n.value + 1)
        assert self.lib.trax_physics_csv(self.h, what, lt, buf, n.value + 1, C.byref(n)) == 0
        return buf.value.decode()

    def __del__(self):
        self.lib.trax_physics_destroy(self.h)


def test_records_merge_and_csv_hand_computed(lib):
    r = Rec(lib)
    # event 0: 4 tracklets (valid, clone, fake, valid), 3 findable, 1 missed
    r.add(0, 0, [4, 2, 1, 1, 0, 1, 3], [0, 1, 2, 0], [-1, -1, 3, 5], [10, 10, 2, 10], [0], [7])
    r.add(1, 0, [0, 0, 0, 0, 0, 0, 0], [], [], [], [], [])
    lines = r.text().splitlines()
    assert lines[0] == "layerTriplet n eff effVar fr frVar cr crVar"
    # eff 2/3 and 0 -> mean 1/3, var 2/9; fr, cr 1/4 and 0 -> 0.125, 1/32
    assert lines[1] == "0 2 0.333333 0.471405 0.125 0.176777 0.125 0.176777"
    assert lines[2] == "2 2 0.333333 0.471405 0.125 0.176777 0.125 0.176777"
    eta = r.text(1, 0).splitlines()
    assert eta[0].startswith("bin valid fake clones missed misc efficiencyMean")
    assert eta[1:] == ["-0.1 1 0 1 0 0 1 0 0 0 0.5 0", "0 0 0 0 1 0 0 0 0 0 0 0",
                       "0.3 0 1 0 0 0 0 0 1 0 0 0", "0.5 1 0 0 0 0 1 0 0 0 0 0"]
    pt = r.text(2, 2).splitlines()  # the total's pt histogram
    assert pt[1:] == ["0.2 0 1 0 0 0 0 0 1 0 0 0", "0.7 0 0 0 1 0 0 0 0 0 0 0",
                      "1 2 0 1 0 0 1 0 0 0 0.333333 0"]


def load_reference_config():
    """configs/layerTriplets.xml rows and the CMS geometry of
    detectorRadius.dat / radiusDictionary.dat."""
    import xml.etree.ElementTree as ET
    rows = []
    for lt in ET.parse(REF + "/configs/layerTriplets.xml").getroot():
        g = lambda k: lt.find(k).text
        rows.append((int(g("layer1")), int(g("layer2")), int(g("layer3")), float(g("dThetaCut")),
                     float(g("sigmaZ")), float(g("dPhiCut")), float(g("sigmaPhi")),
                     float(g("tipCut")), int(g("pairSpreadZ")), float(int(g("z0"))),
                     int(g("pairSpreadPhi")), int(g("nCandidates"))))
    geo = ingest.load_geometry(REF + "/configs/detectorRadius.dat",
                               REF + "/configs/radiusDictionary.dat")
    return rows, geo


@pytest.mark.skipif(not os.path.exists(TTBAR), reason="reference checkout not present")
def test_ttbar_chain_through_oracle(lib):
    """hits.ttBar.pb -> addEvent -> seeding -> physics, all on the oracle,
    with the reference's ttBar.reco.conf settings (minPt 1, 50 x 8 grid, 4
    layer triplets).  Efficiency must be physical (the reference's table for
    its larger ttbar sample reads 0.74-0.84)."""
    rows, geo = load_reference_config()
    cfg = make_config(rows, geo.min_radius, geo.max_radius, 1.0)
    assert geo.min_radius[0] == pytest.approx(4.13, abs=1e-3)
    d = ingest.decode(open(TTBAR, "rb").read())
    ml, mask = ingest.used_layers(cfg)
    assert (ml, mask) == (8, 0b10011111)
    idx, ln, trk, toff = oracle.add_events(d.layer, d.sim_track_id, d.sim_track_pt,
                                           d.hit_offset, 1.0, ml, mask)
    ev = np.repeat(np.arange(d.n_events, dtype=np.uint32), ln.sum(axis=1).astype(np.int64))
    b = gen.EventBatch(d.x[idx], d.y[idx], d.z[idx], d.layer[idx], d.detector_id[idx],
                       d.sim_track_id[idx], ev, ln)
    from trax_gb300._abi import TraxGridCfg
    grid = TraxGridCfg(d.n_events, ml, 50, 8)
    r = oracle.run(b, cfg, grid, 4, n_threads=256)
    assert r["stats"]["status"] == 0
    so = r["sorted_orig"]
    T = len(rows)
    ph = oracle.physics(b.hit_id[so], b.x[so], b.y[so], b.z[so],
                        np.stack([r["trk_h1"], r["trk_h2"], r["trk_h3"]], axis=1),
                        r["trk_offsets"], d.n_events, T, (trk, toff), d.x, d.y, d.z)
    cnt = ph["counts"].reshape(d.n_events, T, 7)
    eff = cnt[:, :, 1].sum(axis=0) / cnt[:, :, 6].sum(axis=0)
    assert (cnt[:, :, 6] > 0).all()
    # 0.785 for triplet (1,2,3) on these 10 events; the reference's table
    # gives 0.789 on its 200-event sample
    assert 0.7 < eff[0] < 0.9 and 0.5 < eff[1] <= 1.0, eff
    # feed the records into PhysicsRecords and read the table back
    rec = Rec(lib)
    M = len(trk)
    for e in range(d.n_events):
        for lt in range(T):
            g = e * T + lt
            t0, t1 = int(r["trk_offsets"][g]), int(r["trk_offsets"][g + 1])
            ks = [lt * M + k for k in range(int(toff[e]), int(toff[e + 1]))
                  if ph["missed"][lt * M + k]]
            rec.add(e, lt, cnt[e, lt], ph["cat"][t0:t1], ph["eta_bin"][t0:t1],
                    ph["pt_bin"][t0:t1], ph["miss_eta_bin"][ks], ph["miss_pt_bin"][ks])
    lines = rec.text().splitlines()
    assert len(lines) == 1 + T + 1
    for lt in range(T):
        f = lines[1 + lt].split()
        assert int(f[0]) == lt and int(f[1]) == d.n_events
        per_event = cnt[:, lt, 1] / np.maximum(cnt[:, lt, 6], 1)
        assert float(f[2]) == pytest.approx(per_event.mean(), rel=1e-5)
