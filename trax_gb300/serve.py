"""Continuous-batching server over the C-ABI (trax_server_*).

Server.submit() queues one event; poll() returns finished events; replay()
feeds a whole arrival schedule from a native thread (events borrowed from a
pool).  stats() reports p50/p99 arrival-to-result latency and the sustained
rate.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .gen import EventBatch
from .runtime import TraxError, load_library

U32 = np.uint32


def _event_struct(ev: EventBatch, keep: list):
    if ev.n_events != 1:
        raise ValueError("a request is exactly one event")
    # the detector and hit ids are not read by the server and may be None
    cols = [None if c is None else np.ascontiguousarray(c) for c in ev.columns()]
    ln = np.ascontiguousarray(ev.layer_nhits.reshape(-1), dtype=U32)
    keep.extend(cols + [ln])
    return A.TraxEventBatch(1, ev.n_layers, ev.n_hits,
                            *[None if c is None else c.ctypes.data for c in cols], ln.ctypes.data)


class Server:
    def __init__(self, cfg: A.TraxConfig, n_layers, n_sectors_z, n_sectors_phi, slots=2,
                 max_batch_events=256, max_event_hits=200_000, memory_budget_bytes=8 << 30,
                 keep_results=True, device=0, max_batch_hits=0, pairs_per_hit=0,
                 candidates_per_hit=0, tracklets_per_hit=0, tuning=None):
        """tuning: (run_walk, index_min, pair_record[, blocks_per_sm]) for
        every slot, e.g. the autotuner's pick for the stream's density class
        (autotune.tuning_for); None keeps the default."""
        self.lib = load_library()
        self.T = cfg.n_layer_triplets
        tn = A.TraxTuning(*[int(v) for v in tuning]) if tuning else A.TraxTuning()
        opts = A.TraxServerOpts(slots, max_batch_events, max_event_hits, n_layers, n_sectors_z,
                                n_sectors_phi, int(memory_budget_bytes), 1 if keep_results else 0,
                                int(max_batch_hits), int(pairs_per_hit), int(candidates_per_hit),
                                int(tracklets_per_hit), tn)
        h = C.c_void_p()
        st = self.lib.trax_server_create(C.byref(h), device, C.byref(cfg), C.byref(opts))
        if st != 0:
            msg = self.lib.trax_ctx_last_error(None)
            raise TraxError(st, "trax_server_create: " + (msg.decode() if msg else ""))
        self.h = h.value
        self._keep = {}
        self._pool = None

    def close(self):
        if self.h:
            self.lib.trax_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def now_ns(self) -> int:
        return int(self.lib.trax_now_ns())

    def submit(self, ev: EventBatch, arrival_ns=0) -> int:
        keep = []
        s = _event_struct(ev, keep)
        t = C.c_uint64()
        st = self.lib.trax_server_submit(self.h, C.byref(s), int(arrival_ns), 0, C.byref(t))
        if st != 0:
            raise TraxError(st, "submit")
        return int(t.value)

    def poll(self, timeout_ms=1000, capacity=1 << 20):
        h = [np.empty(capacity, U32) for _ in range(3)]
        r = A.TraxServerResult()
        r.hit1, r.hit2, r.hit3 = (x.ctypes.data for x in h)
        r.capacity = capacity
        st = self.lib.trax_server_poll(self.h, C.byref(r), int(timeout_ms))
        if st == 3:
            return None
        if st not in (0, 5):
            raise TraxError(st, "poll")
        n = r.n_tracklets
        return {"ticket": r.ticket, "status": r.status, "arrival_ns": r.arrival_ns,
                "start_ns": r.start_ns, "done_ns": r.done_ns, "batch_events": r.batch_events,
                "tracklets": np.stack([x[:n] for x in h], axis=1),
                "offsets": np.array(r.offsets[: self.T + 1], dtype=U32)}

    def replay(self, pool, order, arrival_ns):
        """Submits pool[order[i]] at arrival_ns[i] from a native feeder thread."""
        keep = []
        structs = (A.TraxEventBatch * len(pool))(*[_event_struct(e, keep) for e in pool])
        order = np.ascontiguousarray(order, dtype=U32)
        arr = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        self._pool = (keep, structs, order, arr)
        st = self.lib.trax_server_replay(self.h, structs, order.ctypes.data, arr.ctypes.data,
                                         len(order))
        if st != 0:
            raise TraxError(st, "replay")

    def drain(self, timeout_ms=120_000):
        st = self.lib.trax_server_drain(self.h, int(timeout_ms))
        if st != 0:
            raise TraxError(st, "drain")
        self._pool = None

    def stats(self) -> dict:
        s = A.TraxServerStats()
        self.lib.trax_server_get_stats(self.h, C.byref(s))
        return s.as_dict()

    def reset_stats(self):
        self.lib.trax_server_reset_stats(self.h)


def poisson_arrivals(n, rate_per_s, start_ns, seed=0):
    """Arrival times of a Poisson stream (exponential gaps)."""
    gaps = np.random.default_rng(seed).exponential(1.0 / rate_per_s, n)
    return (start_ns + np.cumsum(gaps) * 1e9).astype(np.uint64)
