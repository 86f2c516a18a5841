"""ctypes driver for oracle/_ref/libtrax_ref.so: the reference's own OpenCL
kernels, compiled for the host by oracle/ref_build.py, run through the
reference's host chain (restated in oracle/ref_host.cpp).

TEST INFRASTRUCTURE ONLY.  It pins the CPU restatement (trax_oracle.c) to
the reference: tests run both on the same inputs and compare every stage's
output; bench.py's reference arm times it.  It builds from the reference
tree, or from an extraction of the kernels made earlier (which travels with
the working tree); with neither, `available()` is False.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from trax_gb300._abi import TraxConfig, TraxGridCfg

from . import ITEMS, STATS, _DTYPES, PAIR_GENERATORS
from . import ref_build

_lib = None
_lock = threading.Lock()

# variant bits (ref_host.cpp ref_run): which of the reference's kernel
# variants run where it picks one by local memory size
GRID_NO_LOCAL_COUNT = 1
GRID_STORE_WRITTEN_LOCAL = 2
GRID_STORE_NO_LOCAL = 4
PAIR_NO_LOCAL_COUNT = 8


def reference_present() -> bool:
    return os.path.isdir(os.path.join(ref_build.DEFAULT_REFERENCE, "src", "algorithms"))


def available() -> bool:
    """The library can be loaded: the reference tree or an earlier
    extraction of its kernels is here to build it from."""
    return reference_present() or os.path.exists(ref_build.INC_PATH)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            ref_build.build()
            L = C.CDLL(ref_build.LIB_PATH)
            L.ref_run.restype = C.c_void_p
            L.ref_run.argtypes = [C.POINTER(TraxConfig), C.POINTER(TraxGridCfg)] + \
                [C.c_void_p] * 7 + [C.c_uint32] + [C.c_void_p] * 3 + \
                [C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_int]
            L.ref_size.restype = C.c_uint64
            L.ref_size.argtypes = [C.c_void_p, C.c_int]
            L.ref_data.restype = C.c_void_p
            L.ref_data.argtypes = [C.c_void_p, C.c_int]
            L.ref_free.argtypes = [C.c_void_p]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def run(batch, cfg: TraxConfig, grid: TraxGridCfg, n_stages=4, n_threads=256, grid_threads=1,
        pair_gen="beamspot", variant=0, workers=1):
    """Runs the reference's kernels on an EventBatch; returns a dict shaped
    like oracle.run's (no sorted_phi / sorted_orig: the reference keeps
    neither; stats["cand_truncated"] is not measured).  grid_threads is the
    grid stage's work-group size: 1 fixes gridStore's racy within-cell order
    to the input order, the order the restatement and the CUDA kernels use.
    workers > 1 runs work-groups on that many threads (timing only: racy
    kernels then give no fixed result)."""
    L = lib()
    cols = [np.ascontiguousarray(c) for c in batch.columns()]
    eo = np.ascontiguousarray(batch.event_offset, dtype=np.uint32)
    ln = np.ascontiguousarray(batch.layer_nhits.reshape(-1), dtype=np.uint32)
    lo = np.ascontiguousarray(batch.layer_offset.reshape(-1), dtype=np.uint32)
    h = L.ref_run(C.byref(cfg), C.byref(grid), *[_ptr(c) for c in cols], batch.n_hits,
                  _ptr(eo), _ptr(ln), _ptr(lo), n_stages, n_threads, grid_threads,
                  PAIR_GENERATORS[pair_gen], variant, workers)
    out = {}
    try:
        for i, name in enumerate(ITEMS):
            if name in ("sorted_phi", "sorted_orig"):
                continue
            n = int(L.ref_size(h, i))
            p = L.ref_data(h, i)
            dt = _DTYPES.get(name, np.uint32)
            if not p or n == 0:
                out[name] = np.zeros(0, dtype=dt)
                continue
            buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(p)
            out[name] = np.frombuffer(bytes(buf), dtype=dt).copy()
    finally:
        L.ref_free(h)
    out["stats"] = dict(zip(STATS, (int(v) for v in out["stats"])))
    for k in ("pairs", "cands"):
        out[k] = out[k].reshape(-1, 2)
    return out
