"""The oracle's pair, prediction and filter stages against numpy
restatements (brute force for the windows).

The reference visits only the grid cells its windows' sector ranges cover
(PairGeneratorBeamspot.h:172-230, TripletThetaPhiPredictor.h:170-233 and
:379-456).  These tests compute the same windows in numpy float32 (the
project's acos/atan for the transcendentals, the reference's operation
order), test EVERY hit of the event's target layer against them, and check:
- the pair set equals the oracle's (no accepted hit lies outside the
  visited cells);
- per pair, the prediction's count window A and store window B accept the
  oracle's numbers, and the stored candidates are the first min(A, B)
  window-B accepts in the reference's visit order: z row, then (with
  wrap-around) the cells from phiLowSector to the row end before those from
  the row start, then position;
- the filter's cuts, restated from the kernel text, accept exactly the
  oracle's tracklets.
"""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen

F = np.float32
PI = F(np.pi)  # the float nearest to pi
CASES = [("single-muon-100trk", 3), ("multimuon-1000trk", 2), ("pileup50-batch100", 1)]


def _acos(v):
    return oracle.math_batch(1, np.asarray(v, F))


def _atan(v):
    return oracle.math_batch(2, np.asarray(v, F))


def _maxf(x, y):
    """OpenCL max(): y if x < y, otherwise x."""
    return np.where(x < y, y, x)


def _wrap_phi(lo, hi):
    wrap = (lo < -PI) | (hi > PI) | (lo > PI) | (hi < -PI)
    lo = lo - F(2) * PI * (lo > PI)
    lo = lo + F(2) * PI * (lo < -PI)
    hi = hi - F(2) * PI * (hi > PI)
    hi = hi + F(2) * PI * (hi < -PI)
    return lo, hi, wrap


def _in_phi(lo, hi, wrap, phi):
    inw = (lo[:, None] <= phi) & (phi <= hi[:, None])
    inww = ((lo[:, None] <= phi) & (phi <= PI)) | ((-PI <= phi) & (phi <= hi[:, None]))
    return np.where(wrap[:, None], inww, inw)


def _run(name, n_ev, stages):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    cfg = w.config()
    r = oracle.run(b, cfg, w.grid(n_ev), n_stages=stages, n_threads=256)
    assert r["stats"]["status"] == 0
    rminc = F(oracle.lib().or_min_radius_curvature(F(cfg.min_pt), F(cfg.bz)))
    return w, cfg, r, rminc


@pytest.mark.parametrize("name,n_ev", CASES)
def test_pair_set_equals_brute_force(name, n_ev):
    w, cfg, r, rminc = _run(name, n_ev, 2)
    X, Y, Z, PHI = r["sorted_x"], r["sorted_y"], r["sorted_z"], r["sorted_phi"]
    LAY, EV = r["sorted_layer"].astype(np.int64), r["sorted_event"].astype(np.int64)
    got = set(map(tuple, r["pairs"][r["pair_valid"].astype(bool)].tolist()))
    want = set()
    for t in range(cfg.n_layer_triplets):
        lt = cfg.triplets[t]
        l1, l2 = lt.layer1, lt.layer2
        z0, tip, sZ = F(lt.z0), F(lt.tip_cut), F(lt.sigma_z)
        # the host binds the pairSpreadPhi uint as gSigmaPhi: its bits as a float
        sP = np.array([lt.pair_spread_phi], np.uint32).view(F)[0]
        rmin, rmax = F(cfg.min_radius[l1 - 1]), F(cfg.max_radius[l1 - 1])
        for e in range(n_ev):
            o = np.nonzero((EV == e) & (LAY == l2))[0]
            inner = np.nonzero((EV == e) & (LAY == l1))[0]
            x, y, z = X[o], Y[o], Z[o]
            sgn = np.sign(y).astype(F)
            rr = sgn * np.sqrt(x * x + y * y)
            c_hi = (z - z0) / rr
            c_lo = (z + z0) / rr
            tmp = sgn * rmax * c_hi + z0
            z_hi = sgn * rmin * c_hi + z0
            z_hi = F(tmp < z_hi) * z_hi + F(tmp > z_hi) * tmp
            tmp = sgn * rmax * c_lo - z0
            z_lo = sgn * rmin * c_lo - z0
            z_lo = F(tmp < z_lo) * tmp + F(tmp > z_lo) * z_lo
            z_lo = z_lo - sZ
            z_hi = z_hi + sZ
            a0 = _acos(rr / (F(2) * rminc))
            tmp = np.abs(a0 - _acos(rmax / (F(2) * rminc)))
            d_phi = np.abs(a0 - _acos(rmin / (F(2) * rminc)))
            d_phi = F(tmp < d_phi) * d_phi + F(tmp > d_phi) * tmp
            tmp = _atan(tip * (rr - rmin)) / (rr * rmin)
            p_hi = _atan(tip * (rr - rmax)) / (rr * rmax)
            d_phi = d_phi + np.where(tmp > p_hi, tmp, p_hi)
            p_lo, p_hi, wrap = _wrap_phi(PHI[o] - d_phi - sP, PHI[o] + d_phi + sP)
            zi = Z[inner][None, :]
            ok = (z_lo[:, None] <= zi) & (zi <= z_hi[:, None]) & \
                _in_phi(p_lo, p_hi, wrap, PHI[inner][None, :])
            a, c = np.nonzero(ok)
            want |= set(zip(inner[c].tolist(), o[a].tolist()))
    assert got == want


@pytest.mark.parametrize("name,n_ev", CASES)
def test_prediction_equals_brute_force(name, n_ev):
    w, cfg, r, rminc = _run(name, n_ev, 3)
    nz, nphi = w.n_sectors_z, w.n_sectors_phi
    X, Y, Z, PHI = r["sorted_x"], r["sorted_y"], r["sorted_z"], r["sorted_phi"]
    LAY, EV = r["sorted_layer"].astype(np.int64), r["sorted_event"].astype(np.int64)
    pairs, pv = r["pairs"], r["pair_valid"].astype(bool)
    got = {}
    for gid, h3 in r["cands"][r["cand_valid"].astype(bool)].tolist():
        got.setdefault(gid, []).append(h3)
    sz_z = F(F(300.0) - F(-300.0)) / F(nz)
    sz_phi = F(PI - F(-PI)) / F(nphi)
    zsec = np.floor((Z - F(-300.0)) / sz_z).astype(np.int64)
    psec = np.floor((PHI - F(-PI)) / sz_phi).astype(np.int64)
    gids = np.nonzero(pv)[0]
    h1, h2 = pairs[gids, 0].astype(np.int64), pairs[gids, 1].astype(np.int64)
    lt_of, ev_of = LAY[h1] - 1, EV[h1]
    want, slots, truncated = {}, 0, 0
    for t in range(cfg.n_layer_triplets):
        tr = cfg.triplets[t]
        l3 = tr.layer3 - 1
        sZ, sP = F(tr.sigma_z), F(tr.sigma_phi)
        rmin, rmax = F(cfg.min_radius[l3]), F(cfg.max_radius[l3])
        for e in range(n_ev):
            sel = np.nonzero((lt_of == t) & (ev_of == e))[0]
            if not len(sel):
                continue
            third = np.nonzero((EV == e) & (LAY == l3 + 1))[0]
            p1x, p1y, p1z = X[h1[sel]], Y[h1[sel]], Z[h1[sel]]
            p2x, p2y, p2z = X[h2[sel]], Y[h2[sel]], Z[h2[sel]]
            dx, dy = p2x - p1x, p2y - p1y
            tip2 = p1y * dx - p1x * dy
            tip2 = tip2 * tip2
            tip2 = tip2 / (dx * dx + dy * dy)
            windows = []
            for store in (0, 1):
                if store:
                    r1 = np.sqrt(p1x * p1x + p1y * p1y)
                    r_o = np.sqrt(r1 * r1 - tip2)
                else:
                    r_o = np.sqrt((p1x * p1x + p1y * p1y) - tip2)
                cot = (p2z - p1z) / (np.sqrt(p2x * p2x + p2y * p2y - tip2) - r_o)
                tmp = p1z + (np.sqrt(rmax * rmax - tip2) - r_o) * cot
                z_lo = p1z + (np.sqrt(rmin * rmin - tip2) - r_o) * cot
                z_hi = F(tmp > z_lo) * tmp + F(tmp < z_lo) * z_lo
                z_lo = F(tmp > z_lo) * z_lo + F(tmp < z_lo) * tmp
                z_lo = z_lo - sZ
                z_hi = z_hi + (sZ if store else sP)
                zls = np.maximum(np.floor((z_lo - F(-300.0)) / sz_z).astype(np.int64), 0)
                zhs = np.minimum(np.floor((z_hi - F(-300.0)) / sz_z).astype(np.int64) + 1, nz)
                phi = PHI[h2[sel]]
                d_phi = phi - PHI[h1[sel]]
                d_phi = d_phi + np.where(d_phi > PI, F(-2) * PI,
                                         np.where(d_phi < -PI, F(2) * PI, F(0)))
                d_phi = np.abs(d_phi)
                d_hits = np.sqrt(dx * dx + dy * dy)
                a0 = _acos(d_hits / (F(2) * rminc))
                tmp = np.abs(a0 - _acos(rmax / (F(2) * rminc)))
                p_lo = np.abs(a0 - _acos(rmin / (F(2) * rminc)))
                d_phi = _maxf(d_phi, _maxf(tmp, p_lo))
                p_lo, p_hi, wrap = _wrap_phi(phi - d_phi - sP, phi + d_phi + sP)
                pls = np.floor((p_lo - F(-PI)) / sz_phi).astype(np.int64)
                phs = np.minimum(np.floor((p_hi - F(-PI)) / sz_phi).astype(np.int64) + 1, nphi)
                zi = Z[third][None, :]
                ok = (z_lo[:, None] <= zi) & (zi <= z_hi[:, None]) & \
                    _in_phi(p_lo, p_hi, wrap, PHI[third][None, :])
                # every accepted hit lies in a cell the reference visits
                zs3, ps3 = zsec[third][None, :], psec[third][None, :]
                rows = (zs3 >= zls[:, None]) & (zs3 < zhs[:, None])
                cells = np.where(wrap[:, None], (ps3 >= pls[:, None]) | (ps3 < phs[:, None]),
                                 (ps3 >= pls[:, None]) & (ps3 < phs[:, None]))
                assert not (ok & ~(rows & cells)).any()
                windows.append((ok, wrap, pls))
            ok_a, (ok_b, wrap_b, pls_b) = windows[0][0], windows[1]
            count_a = ok_a.sum(axis=1)
            slots += int(count_a.sum())
            for k in range(len(sel)):
                hits = third[np.nonzero(ok_b[k])[0]]
                second_run = (wrap_b[k] & (psec[hits] < pls_b[k])).astype(np.int64)
                hits = hits[np.lexsort((hits, second_run, zsec[hits]))]
                m = min(int(count_a[k]), len(hits))
                truncated += len(hits) - m
                if m:
                    want[int(gids[sel[k]])] = hits[:m].tolist()
    assert slots == r["stats"]["cand_slots"]
    assert truncated == r["stats"]["cand_truncated"]
    assert got == want


def _atan2(y, x):
    return oracle.math_batch(0, np.asarray(y, F), np.asarray(x, F))


@pytest.mark.parametrize("name,n_ev", CASES)
def test_filter_equals_numpy_restatement(name, n_ev):
    """filterCount (TripletThetaPhiFilter.h:50-168) restated in numpy from
    the kernel text -- dTheta ratio, dPhi with wrap fix, the circle fit on the
    paraboloid (normalize(v) = v / sqrt(dot(v, v)), the project's reading of
    the OpenCL built-in), TIP and minimum radius -- applied to every oracle
    candidate: the accepted candidates, in candidate order, are the oracle's
    tracklets, and each (event, layer triplet) offset counts the accepted
    candidates before the group's first candidate."""
    w, cfg, r, rminc = _run(name, n_ev, 4)
    X, Y, Z = r["sorted_x"], r["sorted_y"], r["sorted_z"]
    LAY = r["sorted_layer"].astype(np.int64)
    cv = r["cand_valid"].astype(bool)
    cands, pairs = r["cands"], r["pairs"]
    h1 = pairs[cands[:, 0], 0].astype(np.int64)
    h2 = pairs[cands[:, 0], 1].astype(np.int64)
    h3 = cands[:, 1].astype(np.int64)
    lt = LAY[h1] - 1
    d_theta = np.array([cfg.triplets[t].dtheta_cut for t in range(cfg.n_layer_triplets)], F)[lt]
    d_phi_cut = np.array([cfg.triplets[t].dphi_cut for t in range(cfg.n_layer_triplets)], F)[lt]
    tip_cut = np.array([cfg.triplets[t].tip_cut for t in range(cfg.n_layer_triplets)], F)[lt]
    x1, y1, z1, x2, y2, z2, x3, y3, z3 = X[h1], Y[h1], Z[h1], X[h2], Y[h2], Z[h2], X[h3], Y[h3], Z[h3]
    a1 = _atan2(np.sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)), z2 - z1)
    a2 = _atan2(np.sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2)), z3 - z2)
    delta = np.abs(a2 / a1)
    valid = (F(1) - d_theta <= delta) & (delta <= F(1) + d_theta)
    a1 = _atan2(y2 - y1, x2 - x1)
    a2 = _atan2(y3 - y2, x3 - x2)
    delta = a2 - a1
    delta = delta + np.where(delta > PI, F(-2) * PI, np.where(delta < -PI, F(2) * PI, F(0)))
    valid &= np.abs(delta) <= d_phi_cut
    p1z, p2z, p3z = x1 * x1 + y1 * y1, x2 * x2 + y2 * y2, x3 * x3 + y3 * y3
    ax, ay, az = x2 - x1, y2 - y1, p2z - p1z
    bx, by, bz = x3 - x1, y3 - y1, p3z - p1z
    nx, ny, nz = ay * bz - az * by, az * bx - ax * bz, ax * by - ay * bx
    nlen = np.sqrt(nx * nx + ny * ny + nz * nz)
    nx, ny, nz = nx / nlen, ny / nlen, nz / nlen
    cox, coy = (-nx) / (F(2) * nz), (-ny) / (F(2) * nz)
    c = -(nx * x1 + ny * y1 + nz * p1z)
    c_r = np.sqrt((F(1) - nz * nz - F(4) * c * nz) / (F(4) * nz * nz))
    vx, vy = -cox, -coy
    vlen = np.sqrt(vx * vx + vy * vy)
    vx, vy = vx / vlen, vy / vlen
    pcx, pcy = cox + c_r * vx, coy + c_r * vy
    tip = pcx * pcx + pcy * pcy
    valid &= tip <= tip_cut * tip_cut
    valid &= c_r >= rminc
    valid &= cv
    trk = np.stack([h1[valid], h2[valid], h3[valid]], axis=1)
    got = np.stack([r["trk_h1"], r["trk_h2"], r["trk_h3"]], axis=1).astype(np.int64)
    assert np.array_equal(got, trk)
    before = np.concatenate([[0], np.cumsum(valid)])
    assert np.array_equal(r["trk_offsets"].astype(np.int64), before[r["cand_offsets"]])
