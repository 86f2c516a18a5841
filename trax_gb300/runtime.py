"""ctypes binding of libtrax_gb300.so (include/trax.h).

There is no CPU fallback: if the native library is missing or no CUDA device
is present, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtrax_gb300.so")


class TraxError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = int(status)
        super().__init__(f"{A.STATUS_NAMES.get(self.status, self.status)}: {msg}")


_lib = None
_lock = threading.Lock()

_SIGS = {
    "trax_version": (C.c_char_p, []),
    "trax_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "trax_ctx_destroy": (None, [C.c_void_p]),
    "trax_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "trax_ctx_get_stream": (C.c_void_p, [C.c_void_p]),
    "trax_ctx_last_error": (C.c_char_p, [C.c_void_p]),
    "trax_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "trax_ctx_sm_count": (C.c_int, [C.c_void_p]),
    "trax_configure": (C.c_int, [C.c_void_p, C.POINTER(A.TraxConfig)]),
    "trax_min_radius_curvature": (C.c_float, [C.c_float, C.c_float]),
    "trax_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(A.TraxTuning)]),
    "trax_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(A.TraxTuning)]),
    "trax_set_pair_generator": (C.c_int, [C.c_void_p, C.c_int]),
    "trax_get_pair_generator": (C.c_int, [C.c_void_p]),
    "trax_dev_alloc": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_size_t]),
    "trax_dev_free": (C.c_int, [C.c_void_p, C.c_void_p]),
    "trax_host_alloc_pinned": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_size_t]),
    "trax_host_free_pinned": (C.c_int, [C.c_void_p, C.c_void_p]),
    "trax_memcpy_h2d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "trax_memcpy_d2h": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "trax_memset_d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_size_t]),
    "trax_timer_record": (C.c_int, [C.c_void_p, C.c_int]),
    "trax_timer_elapsed_ms": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "trax_grid_build": (C.c_int, [C.c_void_p, C.POINTER(A.TraxHits), C.POINTER(A.TraxLayout),
                                  C.POINTER(A.TraxGridCfg), C.POINTER(A.TraxSortedHits),
                                  C.c_void_p]),
    "trax_pair_gen": (C.c_int, [C.c_void_p, C.POINTER(A.TraxSortedHits), C.c_void_p,
                                C.POINTER(A.TraxGridCfg), C.POINTER(A.TraxPairs)]),
    "trax_pb_scan": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int, C.POINTER(C.c_uint32),
                               C.POINTER(C.c_uint64)]),
    "trax_pb_decode": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int, C.POINTER(A.TraxPbEvents),
                                 C.c_int]),
    "trax_pb_error": (C.c_char_p, []),
    "trax_ingest": (C.c_int, [C.c_void_p, C.POINTER(A.TraxRawHits), C.POINTER(A.TraxIngestCfg),
                              C.c_void_p, C.c_uint32, C.POINTER(A.TraxHitsOut), C.c_void_p,
                              C.POINTER(A.TraxTrackList), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32)]),
    "trax_physics_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "trax_physics_destroy": (None, [C.c_void_p]),
    "trax_physics_n_records": (C.c_uint32, [C.c_void_p]),
    "trax_physics_eval": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(A.TraxSortedHits),
                                    C.POINTER(A.TraxTracklets), C.c_uint32, C.c_uint32,
                                    C.POINTER(A.TraxTrackList), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "trax_physics_add_group": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                         C.c_void_p, C.c_void_p, C.c_uint32]),
    "trax_physics_csv": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_char_p, C.c_size_t,
                                   C.POINTER(C.c_size_t)]),
    "trax_pair_gen_sector": (C.c_int, [C.c_void_p, C.POINTER(A.TraxSortedHits), C.c_void_p,
                                       C.POINTER(A.TraxGridCfg), C.POINTER(A.TraxPairs)]),
    "trax_triplet_predict": (C.c_int, [C.c_void_p, C.POINTER(A.TraxSortedHits), C.c_void_p,
                                       C.POINTER(A.TraxGridCfg), C.POINTER(A.TraxPairs),
                                       C.POINTER(A.TraxPairs)]),
    "trax_triplet_filter": (C.c_int, [C.c_void_p, C.POINTER(A.TraxSortedHits),
                                      C.POINTER(A.TraxGridCfg), C.POINTER(A.TraxPairs),
                                      C.POINTER(A.TraxPairs), C.POINTER(A.TraxTracklets)]),
    "trax_read_counts": (C.c_int, [C.c_void_p, C.POINTER(A.TraxCounts)]),
    "trax_triplet_connectivity": (C.c_int, [C.c_void_p, C.POINTER(A.TraxTracklets), C.c_uint32,
                                            C.c_void_p, C.POINTER(A.TraxTracklets), C.c_uint32,
                                            C.c_void_p, C.c_int, C.c_int]),
    "trax_prefix_sum": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "trax_prefix_sum_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                          C.c_void_p]),
    "trax_prefix_sum_noalloc_error": (C.c_char_p, []),
    "trax_prefix_sum_noalloc_status": (C.c_int, [C.c_void_p]),
    "trax_count_pairs_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "trax_selftest_lookback_timeout": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                                 C.c_uint32]),
    "trax_reset_counts": (C.c_int, [C.c_void_p]),
    "trax_config_validate": (C.c_int, [C.POINTER(A.TraxConfig), C.POINTER(A.TraxGridCfg)]),
    "trax_layout_validate": (C.c_int, [C.POINTER(A.TraxLayout), C.c_uint32]),
    "trax_abi_sizeof": (C.c_size_t, [C.c_char_p]),
    "trax_eval_math": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_uint32]),
    "trax_reserve": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.POINTER(A.TraxGridCfg), C.c_uint32, C.c_uint32, C.c_uint32]),
    "trax_seed_batch": (C.c_int, [C.c_void_p, C.POINTER(A.TraxEventBatch),
                                  C.POINTER(A.TraxBatchResult)]),
    "trax_stage_batch": (C.c_int, [C.c_void_p, C.POINTER(A.TraxEventBatch)]),
    "trax_submit_batch": (C.c_int, [C.c_void_p, C.POINTER(A.TraxEventBatch),
                                    C.POINTER(A.TraxBatchResult), C.POINTER(C.c_uint32)]),
    "trax_wait_batch": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(A.TraxBatchResult)]),
    "trax_run_staged": (C.c_int, [C.c_void_p]),
    "trax_run_staged_eager": (C.c_int, [C.c_void_p]),
    "trax_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "trax_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_char_p),
                                    C.c_int, C.POINTER(C.c_int)]),
    "trax_kernel_launches": (C.c_int, [C.c_void_p]),
    "trax_now_ns": (C.c_uint64, []),
    "trax_server_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(A.TraxConfig),
                                     C.POINTER(A.TraxServerOpts)]),
    "trax_server_destroy": (None, [C.c_void_p]),
    "trax_server_submit": (C.c_int, [C.c_void_p, C.POINTER(A.TraxEventBatch), C.c_uint64, C.c_int,
                                     C.POINTER(C.c_uint64)]),
    "trax_server_replay": (C.c_int, [C.c_void_p, C.POINTER(A.TraxEventBatch), C.c_void_p,
                                     C.c_void_p, C.c_uint32]),
    "trax_server_poll": (C.c_int, [C.c_void_p, C.POINTER(A.TraxServerResult), C.c_int]),
    "trax_server_drain": (C.c_int, [C.c_void_p, C.c_int]),
    "trax_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(A.TraxServerStats)]),
    "trax_server_reset_stats": (C.c_int, [C.c_void_p]),
}

EXPORTED_SYMBOLS = tuple(_SIGS)


def load_library(path: str | None = None):
    """Loads the native library; raises if it is absent (no fallback)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise TraxError(7, f"native library {p} is missing; run trax_gb300.build.build()")
        L = C.CDLL(p)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if path is None:
            _lib = L
        return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class DeviceBuffer:
    """A device allocation owned by a Context."""

    def __init__(self, ctx: "Context", nbytes: int, dtype=np.uint32):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        self.dtype = np.dtype(dtype)
        p = C.c_void_p()
        ctx._check(ctx.lib.trax_dev_alloc(ctx.h, C.byref(p), max(self.nbytes, 16)))
        self.ptr = p.value

    @property
    def size(self):
        return self.nbytes // self.dtype.itemsize

    def upload(self, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.nbytes > self.nbytes:
            raise ValueError("upload larger than buffer")
        self.ctx._check(self.ctx.lib.trax_memcpy_h2d(self.ctx.h, self.ptr, _ptr(a), a.nbytes))
        self.ctx.synchronize_stream()
        return self

    def download(self, count=None, offset=0) -> np.ndarray:
        n = self.size - offset if count is None else int(count)
        out = np.empty(n, dtype=self.dtype)
        if n:
            self.ctx._check(self.ctx.lib.trax_memcpy_d2h(
                self.ctx.h, _ptr(out), self.ptr + offset * self.dtype.itemsize, out.nbytes))
        return out

    def zero(self):
        self.ctx._check(self.ctx.lib.trax_memset_d(self.ctx.h, self.ptr, 0, self.nbytes))
        return self

    def free(self):
        if self.ptr is not None and self.ctx.h:
            self.ctx.lib.trax_dev_free(self.ctx.h, self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedBuffer:
    def __init__(self, ctx: "Context", nbytes: int, dtype=np.uint32):
        self.ctx = ctx
        p = C.c_void_p()
        ctx._check(ctx.lib.trax_host_alloc_pinned(ctx.h, C.byref(p), max(int(nbytes), 16)))
        self.ptr = p.value
        self.nbytes = int(nbytes)
        self.array = np.frombuffer((C.c_char * max(int(nbytes), 16)).from_address(self.ptr),
                                   dtype=np.uint8)[: int(nbytes)].view(dtype)

    def free(self):
        if self.ptr is not None and self.ctx.h:
            self.ctx.lib.trax_host_free_pinned(self.ctx.h, self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One trax_ctx: a device, a stream, scratch and the configured path."""

    def __init__(self, device: int = 0, lib=None):
        self.lib = lib or load_library()
        h = C.c_void_p()
        st = self.lib.trax_ctx_create(C.byref(h), device)
        if st != 0:
            msg = self.lib.trax_ctx_last_error(None)
            raise TraxError(st, "trax_ctx_create failed: " + (msg.decode() if msg else ""))
        self.h = h.value
        self.config = None

    def close(self):
        if self.h:
            self.lib.trax_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            msg = self.lib.trax_ctx_last_error(self.h)
            raise TraxError(st, msg.decode() if msg else "")
        return st

    @property
    def sm_count(self) -> int:
        return int(self.lib.trax_ctx_sm_count(self.h))

    def configure(self, cfg: A.TraxConfig):
        self._check(self.lib.trax_configure(self.h, C.byref(cfg)))
        self.config = cfg
        return self

    def set_tuning(self, run_walk: int, index_min: int, pair_record: int = 3,
                   blocks_per_sm: int = 0):
        self._check(self.lib.trax_set_tuning(
            self.h, C.byref(A.TraxTuning(run_walk, index_min, pair_record, blocks_per_sm))))

    def set_pair_generator(self, name: str):
        """"beamspot" or "sector": the pair generator of the batched pipeline."""
        self._check(self.lib.trax_set_pair_generator(self.h, A.PAIR_GENERATORS[name]))

    def get_tuning(self):
        t = A.TraxTuning()
        self._check(self.lib.trax_get_tuning(self.h, C.byref(t)))
        return int(t.run_walk), int(t.index_min), int(t.pair_record), int(t.blocks_per_sm)

    def alloc(self, n, dtype=np.uint32) -> DeviceBuffer:
        return DeviceBuffer(self, int(n) * np.dtype(dtype).itemsize, dtype)

    def upload(self, arr, dtype=None) -> DeviceBuffer:
        a = np.ascontiguousarray(arr, dtype=dtype or arr.dtype)
        return DeviceBuffer(self, a.nbytes, a.dtype).upload(a)

    def synchronize_stream(self):
        st = self.lib.trax_ctx_synchronize(self.h)
        if st not in (0,) and st == 4:
            self._check(st)
        return st

    def synchronize(self):
        """Waits for the stream; raises on a device-side fault."""
        return self._check(self.lib.trax_ctx_synchronize(self.h))

    def counts(self) -> dict:
        c = A.TraxCounts()
        self._check(self.lib.trax_read_counts(self.h, C.byref(c)))
        return c.as_dict()

    def reset_counts(self):
        self._check(self.lib.trax_reset_counts(self.h))

    def prefix_sum(self, d_in: DeviceBuffer, d_out: DeviceBuffer, n: int, d_total=None):
        """Exclusive scan of n uint32 on the device (PrefixSum::run)."""
        self._check(self.lib.trax_prefix_sum(self.h, d_in.ptr, d_out.ptr, int(n),
                                             d_total.ptr if d_total is not None else None))

    def timer_record(self, slot):
        self._check(self.lib.trax_timer_record(self.h, slot))

    def timer_elapsed_ms(self, a, b) -> float:
        ms = C.c_float()
        self._check(self.lib.trax_timer_elapsed_ms(self.h, a, b, C.byref(ms)))
        return float(ms.value)
