"""The oracle's grid build against an independent numpy restatement of
GridBuilder (GridBuilder.cpp:6-160, gridCount/gridStore in GridBuilder.h):
each hit's cell is floor((z - MIN_Z) / sectorSizeZ) * (nPhi + 1) +
floor((phi - MIN_PHI) / sectorSizePhi) in float32, phi the project's atan2,
and the sorted order is a stable sort by (event, layer, cell) -- hits keep
their input order inside a cell.  The cell starts are the exclusive prefix
of the cell counts over the whole batch."""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300._abi import TraxGridCfg, make_config

F = np.float32
PI = F(np.pi)  # the float nearest to pi, as the project's M_PI_F


def numpy_grid(b, n_sectors_z, n_sectors_phi):
    P1 = n_sectors_phi + 1
    C = (n_sectors_z + 1) * P1
    phi = oracle.math_batch(0, b.y, b.x)  # the project atan2, bit for bit
    sz_z = F(F(300.0) - F(-300.0)) / F(n_sectors_z)
    sz_phi = F(PI - F(-PI)) / F(n_sectors_phi)
    zs = np.floor((b.z - F(-300.0)) / sz_z).astype(np.int64)
    ps = np.floor((phi - F(-PI)) / sz_phi).astype(np.int64)
    assert zs.min(initial=0) >= 0 and zs.max(initial=0) <= n_sectors_z
    assert ps.min(initial=0) >= 0 and ps.max(initial=0) <= n_sectors_phi
    seg = b.event.astype(np.int64) * b.n_layers + (b.layer.astype(np.int64) - 1)
    key = seg * C + zs * P1 + ps
    order = np.argsort(key, kind="stable")
    counts = np.bincount(key, minlength=b.n_events * b.n_layers * C)
    grid = (np.cumsum(counts) - counts).astype(np.uint32)
    return order.astype(np.uint32), grid, phi


def _check(b, cfg, nz, nphi):
    r = oracle.run(b, cfg, TraxGridCfg(b.n_events, b.n_layers, nz, nphi), n_stages=1,
                   n_threads=256)
    assert r["stats"]["status"] == 0
    order, grid, phi = numpy_grid(b, nz, nphi)
    assert np.array_equal(r["sorted_orig"], order)
    assert np.array_equal(r["grid"], grid)
    assert np.array_equal(r["sorted_phi"].view(np.uint32), phi[order].view(np.uint32))
    for col in ("x", "y", "z"):
        assert np.array_equal(r["sorted_" + col].view(np.uint32),
                              getattr(b, col)[order].view(np.uint32))


@pytest.mark.parametrize("name,n_ev", [("single-muon-100trk", 3), ("multimuon-1000trk", 3),
                                       ("pileup50-batch100", 1)])
def test_oracle_grid_equals_numpy_restatement(name, n_ev):
    w = gen.WORKLOADS[name]
    b = gen.generate_batch(w, n_ev)
    _check(b, w.config(), w.n_sectors_z, w.n_sectors_phi)


def test_cell_boundaries_and_phi_extremes():
    """Hits exactly on z sector boundaries (both grid ends included), at
    phi = +-pi and on phi sector boundaries: the restatement and the oracle
    put every hit in the same cell and order."""
    nz, nphi = 8, 16
    sz_z = F(600.0) / F(nz)
    zs = [F(-300.0) + F(k) * sz_z for k in range(nz + 1)]
    zs += [np.nextafter(z, F(-1e9)) for z in zs[1:]] + [np.nextafter(z, F(1e9)) for z in zs[:-1]]
    angles = [F(k) * (F(2) * PI / F(nphi)) - PI for k in range(nphi + 1)]
    pts = []
    for z in zs:
        for a in angles:
            r = F(7.3)
            pts.append((F(r * np.cos(a)), F(r * np.sin(a)), F(z)))
    pts += [(F(-7.3), F(0.0), F(0.0)), (F(-7.3), F(-0.0), F(1.0))]  # phi = +pi and -pi
    x, y, z = (np.array(c, np.float32) for c in zip(*pts))
    n = len(x)
    b = gen.EventBatch(x, y, z, np.ones(n, np.uint32), np.zeros(n, np.uint32),
                       np.arange(n, dtype=np.uint32), np.zeros(n, np.uint32),
                       np.array([[n]], np.uint32))
    row = (1, 1, 1, 0.01, 0.037, 0.02, 0.032, 0.5, 2, 10.0, 2, 4)
    cfg = make_config([row], (7.0,), (7.6,), 1.0)
    _check(b, cfg, nz, nphi)
