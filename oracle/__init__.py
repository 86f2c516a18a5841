"""ctypes driver for the CPU oracle (trax_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py use it as the checker.  Parity status: pinned to the
reference's own kernels (oracle/ref.py, tests/test_ref_pin.py; see
trax_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from trax_gb300._abi import TraxConfig, TraxGridCfg

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtrax_oracle.so")

ITEMS = ("sorted_x", "sorted_y", "sorted_z", "sorted_phi", "sorted_layer", "sorted_det",
         "sorted_hitid", "sorted_event", "sorted_orig", "grid", "pairs", "pair_valid",
         "pair_offsets", "cands", "cand_valid", "cand_offsets", "trk_h1", "trk_h2", "trk_h3",
         "trk_offsets", "stats")
_DTYPES = {"sorted_x": np.float32, "sorted_y": np.float32, "sorted_z": np.float32,
           "sorted_phi": np.float32, "pair_valid": np.uint8, "cand_valid": np.uint8,
           "stats": np.uint64}
STATS = ("status", "detail", "pair_slots", "pairs", "cand_slots", "cands", "cand_truncated",
         "tracklets")

_lib = None
_lock = threading.Lock()


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = C.CDLL(LIB_PATH)
            L.or_run.restype = C.c_void_p
            L.or_run.argtypes = [C.POINTER(TraxConfig), C.POINTER(TraxGridCfg)] + [C.c_void_p] * 7 + \
                [C.c_uint32] + [C.c_void_p] * 3 + [C.c_int, C.c_uint32, C.c_int]
            L.or_run_ex.restype = C.c_void_p
            L.or_run_ex.argtypes = L.or_run.argtypes + [C.c_int]
            L.or_size.restype = C.c_uint64
            L.or_size.argtypes = [C.c_void_p, C.c_int]
            L.or_data.restype = C.c_void_p
            L.or_data.argtypes = [C.c_void_p, C.c_int]
            L.or_free.argtypes = [C.c_void_p]
            L.or_prefix_sum.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32]
            for f in ("or_atan2f",):
                getattr(L, f).restype = C.c_float
                getattr(L, f).argtypes = [C.c_float, C.c_float]
            for f in ("or_acosf", "or_atanf"):
                getattr(L, f).restype = C.c_float
                getattr(L, f).argtypes = [C.c_float]
            L.or_math_batch.restype = None
            L.or_math_batch.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]
            L.or_connectivity.restype = None
            L.or_connectivity.argtypes = [C.c_void_p] * 4 + [C.c_uint32] + [C.c_void_p] * 4 + \
                [C.c_uint32, C.c_int, C.c_int]
            L.or_connectivity_literal_wide.restype = None
            L.or_connectivity_literal_wide.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32,
                                                       C.c_void_p, C.c_void_p, C.c_uint32]
            L.or_add_event.restype = C.c_uint32
            L.or_add_event.argtypes = [C.c_void_p] * 3 + [C.c_uint32, C.c_uint32, C.c_float,
                                                          C.c_uint32, C.c_uint32, C.c_int,
                                                          C.c_int32] + [C.c_void_p] * 4
            L.or_physics.restype = None
            L.or_physics.argtypes = [C.c_void_p] * 8 + [C.c_uint32, C.c_uint32] + \
                [C.c_void_p] * 15
            L.or_asinh.restype = C.c_double
            L.or_asinh.argtypes = [C.c_double]
            L.or_floor_div_mismatches.restype = C.c_uint64
            L.or_floor_div_mismatches.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
            L.or_min_radius_curvature.restype = C.c_float
            L.or_min_radius_curvature.argtypes = [C.c_float, C.c_float]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def math_batch(fn, a, b=None):
    """fn 0: atan2(a, b), 1: acos(a), 2: atan(a) with the project FP32 math;
    3 / 4: the float-to-uint / float-to-int casts (result bits as float32)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    bb = np.ascontiguousarray(b if b is not None else a, dtype=np.float32)
    out = np.empty_like(a)
    lib().or_math_batch(fn, _ptr(a), _ptr(bb), _ptr(out), a.size)
    return out


def prefix_sum(values, wg):
    a = np.ascontiguousarray(values, dtype=np.uint32).copy()
    lib().or_prefix_sum(_ptr(a), a.size, wg)
    return a


PAIR_GENERATORS = {"beamspot": 0, "sector": 1}


def run(batch, cfg: TraxConfig, grid: TraxGridCfg, n_stages=4, n_threads=256, omp_threads=1,
        pair_gen="beamspot"):
    """Runs the oracle on an EventBatch; returns a dict of numpy arrays.
    pair_gen: "beamspot" (PairGeneratorBeamspot) or "sector"
    (PairGeneratorSector)."""
    L = lib()
    cols = [np.ascontiguousarray(c) for c in batch.columns()]
    eo = np.ascontiguousarray(batch.event_offset, dtype=np.uint32)
    ln = np.ascontiguousarray(batch.layer_nhits.reshape(-1), dtype=np.uint32)
    lo = np.ascontiguousarray(batch.layer_offset.reshape(-1), dtype=np.uint32)
    h = L.or_run_ex(C.byref(cfg), C.byref(grid), *[_ptr(c) for c in cols], batch.n_hits,
                    _ptr(eo), _ptr(ln), _ptr(lo), n_stages, n_threads, omp_threads,
                    PAIR_GENERATORS[pair_gen])
    if not h:
        raise MemoryError("oracle allocation failed")
    out = {}
    try:
        for i, name in enumerate(ITEMS):
            n = int(L.or_size(h, i))
            p = L.or_data(h, i)
            dt = _DTYPES.get(name, np.uint32)
            if not p or n == 0:
                out[name] = np.zeros(0, dtype=dt)
                continue
            buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(p)
            out[name] = np.frombuffer(bytes(buf), dtype=dt).copy()
    finally:
        L.or_free(h)
    out["stats"] = dict(zip(STATS, (int(v) for v in out["stats"])))
    for k in ("pairs", "cands"):
        out[k] = out[k].reshape(-1, 2)
    return out


def canonical(res):
    """Drops unwritten slots; candidates become (hit1, hit2, hit3) rows."""
    pv = res["pair_valid"].astype(bool)
    pairs = res["pairs"][pv] if res["pairs"].size else res["pairs"]
    cv = res["cand_valid"].astype(bool)
    cands = res["cands"][cv] if res["cands"].size else res["cands"]
    full = res["pairs"]
    trip = np.stack([full[cands[:, 0], 0], full[cands[:, 0], 1], cands[:, 1]], axis=1) \
        if cands.size else np.zeros((0, 3), np.uint32)
    trk = np.stack([res["trk_h1"], res["trk_h2"], res["trk_h3"]], axis=1)
    return {"pairs": pairs, "cand_hits": trip, "tracklets": trk}


def connectivity(base, base_con, follow, follow_con, iterate_backwards=False,
                 tight_packing=False):
    """base/follow: (n, 3) hit rows; returns the updated following connectivity."""
    b = np.ascontiguousarray(base, dtype=np.uint32).reshape(-1, 3)
    f = np.ascontiguousarray(follow, dtype=np.uint32).reshape(-1, 3)
    bc = np.ascontiguousarray(base_con, dtype=np.uint32)
    fc = np.ascontiguousarray(follow_con, dtype=np.uint32).copy()
    cols = [np.ascontiguousarray(b[:, i]) for i in range(3)] + \
        [np.ascontiguousarray(f[:, i]) for i in range(3)]
    lib().or_connectivity(_ptr(cols[0]), _ptr(cols[1]), _ptr(cols[2]), _ptr(bc), len(b),
                          _ptr(cols[3]), _ptr(cols[4]), _ptr(cols[5]), _ptr(fc), len(f),
                          int(iterate_backwards), int(tight_packing))
    return fc


def connectivity_literal_wide(base_hit, base_con, follow_hit, follow_con):
    bh = np.ascontiguousarray(base_hit, dtype=np.uint32)
    bc = np.ascontiguousarray(base_con, dtype=np.uint32)
    fh = np.ascontiguousarray(follow_hit, dtype=np.uint32)
    fc = np.ascontiguousarray(follow_con, dtype=np.uint32).copy()
    lib().or_connectivity_literal_wide(_ptr(bh), _ptr(bc), len(bh), _ptr(fh), _ptr(fc), len(fh))
    return fc


def add_events(layer, track, pt, hit_offset, min_pt, max_layer, used_mask, only_tracks=True,
               num_tracks=-1):
    """HitCollection::addEvent over every event of decoded columns.  Returns
    (selected raw indices, layer_nhits [E, max_layer], tracks [(id, inner,
    middle, outer)] as an (n, 4) array, track offsets [E + 1])."""
    layer = np.ascontiguousarray(layer, np.uint32)
    track = np.ascontiguousarray(track, np.uint32)
    pt = np.ascontiguousarray(pt, np.float32)
    off = np.asarray(hit_offset, np.int64)
    E = len(off) - 1
    idx_all, ln_all, trk_all, toff = [], np.zeros((E, max_layer), np.uint32), [], [0]
    for e in range(E):
        n = int(off[e + 1] - off[e])
        out = np.zeros(max(n, 1), np.uint32)
        ln = np.zeros(max_layer, np.uint32)
        trk = np.zeros((max(n, 1), 4), np.uint32)
        nt = C.c_uint32(0)
        w = lib().or_add_event(_ptr(layer), _ptr(track), _ptr(pt), int(off[e]), n,
                               float(min_pt), int(max_layer), int(used_mask), int(only_tracks),
                               int(num_tracks), _ptr(out), _ptr(ln), _ptr(trk), C.byref(nt))
        idx_all.append(out[:w])
        ln_all[e] = ln
        trk_all.append(trk[:nt.value])
        toff.append(toff[-1] + nt.value)
    cat = lambda a, shape: np.concatenate(a) if a else np.zeros(shape, np.uint32)
    return (cat(idx_all, (0,)), ln_all, cat(trk_all, (0, 4)).reshape(-1, 4),
            np.array(toff, np.uint32))


def physics(hid, x, y, z, trk, toff, n_events, n_lt, tracks, rx, ry, rz):
    """PhysicsRecord::fillData per (event, layer triplet).  trk: (K, 3)
    sorted-hit indices; tracks: (M, 4) rows (id, inner, middle, outer) with
    offsets tracks_off in tracks[1].  Returns dict of arrays."""
    mc, moff = tracks
    u = lambda a: np.ascontiguousarray(a, np.uint32)
    f = lambda a: np.ascontiguousarray(a, np.float32)
    trk = u(trk).reshape(-1, 3)
    mc = u(mc).reshape(-1, 4)
    K, M, G = len(trk), len(mc), n_events * n_lt
    cols = [u(trk[:, i]) for i in range(3)] + [u(mc[:, i]) for i in range(4)]
    out = {"counts": np.zeros((G, 7), np.uint32), "cat": np.zeros(max(K, 1), np.uint8),
           "eta_bin": np.zeros(max(K, 1)), "pt_bin": np.zeros(max(K, 1)),
           "missed": np.zeros(max(n_lt * M, 1), np.uint8),
           "miss_eta_bin": np.zeros(max(n_lt * M, 1)), "miss_pt_bin": np.zeros(max(n_lt * M, 1))}
    hid, x, y, z, toff, moff = u(hid), f(x), f(y), f(z), u(toff), u(moff)
    rx, ry, rz = f(rx), f(ry), f(rz)
    lib().or_physics(_ptr(hid), _ptr(x), _ptr(y), _ptr(z), _ptr(cols[0]), _ptr(cols[1]),
                     _ptr(cols[2]), _ptr(toff), n_events, n_lt, _ptr(cols[3]), _ptr(cols[4]),
                     _ptr(cols[5]), _ptr(cols[6]), _ptr(moff), _ptr(rx), _ptr(ry), _ptr(rz),
                     *(_ptr(out[k]) for k in ("counts", "cat", "eta_bin", "pt_bin", "missed",
                                               "miss_eta_bin", "miss_pt_bin")))
    for k in ("cat", "eta_bin", "pt_bin"):
        out[k] = out[k][:K]
    for k in ("missed", "miss_eta_bin", "miss_pt_bin"):
        out[k] = out[k][:n_lt * M]
    return out
