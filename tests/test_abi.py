"""CPU checks of the C-ABI library: it loads, exports every function that
include/trax.h declares, its struct layouts match the ctypes mirror, and the
host-side validation behaves.  No compute call needs a GPU here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import trax_gb300
from trax_gb300 import _abi as A
from trax_gb300 import gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "trax.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(trax_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from trax_gb300 import build
    build.build()
    return trax_gb300.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(names) <= set(trax_gb300.EXPORTED_SYMBOLS)


@pytest.mark.parametrize("name,cls", [
    ("trax_grid_cfg", A.TraxGridCfg), ("trax_layer_triplet", A.TraxLayerTriplet),
    ("trax_tuning", A.TraxTuning),
    ("trax_config", A.TraxConfig), ("trax_hits", A.TraxHits),
    ("trax_sorted_hits", A.TraxSortedHits), ("trax_layout", A.TraxLayout),
    ("trax_pairs", A.TraxPairs), ("trax_tracklets", A.TraxTracklets),
    ("trax_counts", A.TraxCounts), ("trax_event_batch", A.TraxEventBatch),
    ("trax_batch_result", A.TraxBatchResult), ("trax_server_opts", A.TraxServerOpts),
    ("trax_server_result", A.TraxServerResult), ("trax_server_stats", A.TraxServerStats),
    ("trax_pb_events", A.TraxPbEvents), ("trax_raw_hits", A.TraxRawHits),
    ("trax_ingest_cfg", A.TraxIngestCfg), ("trax_hits_out", A.TraxHitsOut),
    ("trax_track_list", A.TraxTrackList)])
def test_struct_layout(lib, name, cls):
    assert lib.trax_abi_sizeof(name.encode()) == C.sizeof(cls)


def test_version_and_no_device(lib):
    assert b"sm_103a" in lib.trax_version()
    assert abs(lib.trax_min_radius_curvature(1.0, 0.0) - 87.522) < 1e-2


def test_config_validation(lib):
    w = gen.WORKLOADS["multimuon-1000trk"]
    cfg = w.config()
    g = w.grid(1)
    assert lib.trax_config_validate(C.byref(cfg), C.byref(g)) == 0
    bad = w.config()
    bad.triplets[1].layer1 = 1  # triplet 1 must start on layer 2
    assert lib.trax_config_validate(C.byref(bad), None) == 1
    bad = w.config()
    bad.triplets[0].layer3 = 9  # no geometry for layer 9
    assert lib.trax_config_validate(C.byref(bad), None) == 1
    small = A.TraxGridCfg(1, 3, 12, 32)  # triplet (2,3,4) outside a 3-layer grid
    assert lib.trax_config_validate(C.byref(cfg), C.byref(small)) == 1
    huge = A.TraxGridCfg(1, 4, 600, 600)
    assert lib.trax_config_validate(C.byref(cfg), C.byref(huge)) == 1
    bad = w.config()
    bad.min_pt = 0.0
    assert lib.trax_config_validate(C.byref(bad), None) == 1


def test_layout_validation(lib):
    b = gen.generate_batch(gen.WORKLOADS["single-muon-100trk"], 3)
    en, eo = b.event_nhits, b.event_offset
    ln, lo = b.layer_nhits.reshape(-1).copy(), b.layer_offset.reshape(-1).copy()

    def check(n_hits, ln=ln, lo=lo, eo=eo):
        lay = A.TraxLayout(b.n_events, b.n_layers, en.ctypes.data, eo.ctypes.data,
                           ln.ctypes.data, lo.ctypes.data)
        return lib.trax_layout_validate(C.byref(lay), n_hits)

    assert check(b.n_hits) == 0
    assert check(b.n_hits + 1) == 6
    lo2 = lo.copy()
    lo2[1] += 1
    assert check(b.n_hits, lo=lo2) == 6
    eo2 = eo.copy()
    eo2[2] -= 1
    assert check(b.n_hits, eo=eo2) == 6


def test_context_without_gpu_fails_loudly(lib):
    import trax_gb300.runtime as R
    h = C.c_void_p()
    st = lib.trax_ctx_create(C.byref(h), 0)
    if st == 0:  # a GPU is present; nothing to check here
        lib.trax_ctx_destroy(h)
        pytest.skip("GPU present")
    assert st == 7
    with pytest.raises(R.TraxError):
        R.Context(0)
