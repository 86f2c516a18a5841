#!/usr/bin/env python3
"""Benchmark of the GB300 triplet-seeding path; prints one JSON line.

A step is one pass of the whole path (grid build -> pairs -> prediction ->
filter) over one batch of synthetic events of the named workload.  The
headline workload is the high-pile-up configuration (Poisson(200) pile-up
vertices, 256 events per step), where the batched-versus-per-event and HBM
targets of this path are set.
  value  events/s with the batch already resident in HBM (CUDA-graph replay)
  e2e    events/s through the streaming API (trax_submit_batch /
         trax_wait_batch) with pinned host buffers: every step uploads the hit
         columns, runs the graph and writes the tracklets back to the host,
         with one step's upload overlapping the previous step's chain (the
         one-at-a-time trax_seed_batch figure is reported beside it)
Also reported: pairs/s and triplets/s, the plain per-event GPU form (one
event per launch sequence, no graph) and the batched/per-event ratio,
per-kernel times and HBM fractions, the dominant kernel's roofline, parity of
the timed batch's tracklets against the CPU oracle, the pile-up-50 batch of
100 events and the multi-muon batch as further sections, the grid autotuner
on pile-up-200 events, the streaming server under Poisson load, the CPU
oracle on all host cores and on one, and SM clocks sampled during the timed
region.

--impl reference times the reference's own kernels compiled for the host
(oracle/_ref: its OpenCL C kernel text built by oracle/ref_build.py, run by a
work-group emulator over all host cores) when that library can be built,
else the CPU restatement of its algorithm, on a bounded sample of the same
workload.

Multi-GPU: replicas only (events are independent).  Under torchrun every
rank runs its own batch; `--gpus N` without torchrun starts N such ranks
itself.  The time is the max over ranks, value = all ranks' events / time.
"""
from __future__ import annotations

import argparse
import json
import os
import socket
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
HEADLINE = "pileup200"
# grid (z x phi bins) each workload is timed at: the workload's own, or for
# the high-pile-up configuration the autotuner's choice (its sweep over
# {8..320} x {16..192} on the full 256-event pile-up-200 batch puts 320 x 192
# first, 0.8 % ahead of 256 x 192; the bench's 'autotune' section repeats the
# sweep on 32 events, where the two trade places within half a percent, and
# reports how far the headline grid is from that sweep's best)
TUNED_GRID = {"pileup200": (320, 192),
              # the streaming mix (pile-up U{0..200}) served at the grid and walk
              # the autotuner picks for its densest events
              "stream-pileup-u200": (256, 192)}
# walk tuning (run_walk, index_min, pair_record) recorded with a tuned grid
TUNED_WALK = {"stream-pileup-u200": (1 << 30, 256, 2)}
# (workload, events per launch) measured beside the headline
SECTIONS = (("pileup50-batch100", 100), ("multimuon-1000trk", 2048))
# capacities per hit (pairs, candidates, tracklets) of the first sizing run
SIZING_CAPS = (48, 96, 8)


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=HEADLINE)
    ap.add_argument("--events", type=int, default=256, help="events per step (batch)")
    ap.add_argument("--per-event-sample", type=int, default=32)
    ap.add_argument("--parity-events", type=int, default=4,
                    help="events of the timed batch checked against the CPU oracle")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sections", action="store_true")
    ap.add_argument("--serve-rates", default="1000,5000,20000,50000",
                    help="Poisson arrival rates (events/s) for the streaming measurement")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-pool", type=int, default=128)
    ap.add_argument("--serve-grid", default="tuned",
                    help="ZxP bins of the serving measurement, 'tuned' or 'workload'")
    ap.add_argument("--serve-walk", default=None,
                    help="run_walk,index_min,pair_record of the serving slots (default: the "
                         "tuned one where a grid is recorded, else the library default)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--autotune-events", type=int, default=32)
    ap.add_argument("--walk", default=None,
                    help="run_walk,index_min,pair_record instead of tuning them on the batch")
    ap.add_argument("--only-resident", action="store_true",
                    help="time only the resident graph replays (for profiler runs)")
    ap.add_argument("--grid", default="tuned",
                    help="ZxP bins, 'tuned' (the autotuned grid where one is recorded) "
                         "or 'workload' (the workload's own)")
    return ap.parse_args(argv)


def workload_at_grid(w, spec):
    """The workload `w` at the grid `spec` names."""
    from trax_gb300 import gen
    if spec == "workload" or (spec == "tuned" and w.name not in TUNED_GRID):
        return w
    z, p = TUNED_GRID[w.name] if spec == "tuned" else map(int, spec.lower().split("x"))
    return gen.Workload(w.name, w.config_id, w.n_layers, w.noise, w.pt_range, z, p,
                        w.n_triplets, tracks=w.tracks, pileup_mean=w.pileup_mean,
                        pileup_uniform=w.pileup_uniform, cut_override=w.cut_override,
                        events=w.events)


# --------------------------------------------------------------------------
# distributed plumbing (host side only: barrier and max over ranks)

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def replica_first_event(rank: int, events_per_rank: int) -> int:
    """Replicas only: rank r seeds events [r*B, (r+1)*B) of the workload."""
    return rank * events_per_rank


def aggregate_rate(dist: "Dist", events_this_rank: int, steps: int, ms_this_rank: float):
    """Whole-job rate: events of all ranks over the slowest rank's time."""
    ms = dist.max(ms_this_rank)
    events = dist.sum(events_this_rank)
    return events * steps / (ms / 1000.0), ms, events


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def launch_replicas(n: int, argv) -> int:
    """`--gpus N` without a launcher: starts N ranks of this script (one per
    GPU, RANK / LOCAL_RANK / WORLD_SIZE set, gloo rendezvous on 127.0.0.1),
    forwards rank 0's output and returns the worst exit code."""
    port = _free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + list(argv),
                                      env=env,
                                      stdout=None if r == 0 else subprocess.DEVNULL))
    return max(abs(p.wait()) for p in procs)


# --------------------------------------------------------------------------
# clocks sampled during the timed region

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, device: int):
        self.proc = None
        self.device = device
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if self.proc is None:
            return None
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------------------
# algorithmic bytes per kernel (traffic a perfect kernel must move)

def layer_sums(b, w):
    ln = b.layer_nhits.astype(np.int64)
    cfg = w.config()
    T = range(cfg.n_layer_triplets)
    return tuple(sum(int(ln[:, getattr(cfg.triplets[t], f"layer{k}") - 1].sum()) for t in T)
                 for k in (1, 2, 3))


def algorithmic_bytes(kernel, b, w, counts):
    """Bytes per launch a kernel must move at least.  grid_build is the
    reference-equivalent figure: xyz read for the cells, the 7 columns read
    and written, the grid counted, scanned and written (68 B/hit)."""
    N = b.n_hits
    E, L = b.n_events, b.n_layers
    C = (w.n_sectors_z + 1) * (w.n_sectors_phi + 1)
    M, K, R = counts["n_pairs"], counts["n_candidates"], counts["n_tracklets"]
    n1, n2, n3 = layer_sums(b, w)
    table = {
        "grid_build": N * (12 + 28 + 28) + E * L * C * 4 * 3,
        # both layers' hits once, the per-outer-hit counts, the pairs
        "pair_gen": 12 * (n1 + n2) + 4 * n2 * 2 + 8 * M,
        # count pass: the pairs and their hits, the layer-3 hits, a count per pair
        "predict": M * (8 + 24) + 12 * n3 + 4 * M,
        # scan of the 32-pair tile totals
        "predict_scan": 8 * ((M + 31) // 32),
        # store pass: a position per pair read, the candidates written
        "predict_store": 4 * M + 8 * K,
        "filter": K * (8 + 8 + 36) + 4 * ((K + 31) // 32) * 3 + 12 * R,
    }
    return table.get(kernel)


def grid_build_actual_bytes(b, w):
    """What the batched chain's grid build itself must move: x, y, z, layer
    and event read once (20 B); layer, event, input position, packed
    (z, phi), half z and (x, y, z, phi) written (38 B); the grid row per
    segment written."""
    E, L = b.n_events, b.n_layers
    C = (w.n_sectors_z + 1) * (w.n_sectors_phi + 1)
    return b.n_hits * (20 + 38) + E * L * C * 4


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def profile_entry(workload, key):
    """An entry of the committed ncu summary (profiles/ncu_traffic.json)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)[workload][key]
    except (OSError, KeyError, ValueError, TypeError):
        return None


# --------------------------------------------------------------------------
# CPU oracle: timing and parity

def oracle_tracklets(batch, w, threads):
    """The oracle's tracklets as input positions, and its offsets.  Work-group
    size 1 puts its pairs -- and so its candidates and tracklets -- in the
    order the CUDA path writes them (outer hit, then inner hit)."""
    import oracle
    r = oracle.run(batch, w.config(), w.grid(batch.n_events), 4, 1, threads)
    so = r["sorted_orig"]
    trk = np.stack([so[r["trk_h1"]], so[r["trk_h2"]], so[r["trk_h3"]]], axis=1) \
        if r["trk_h1"].size else np.zeros((0, 3), np.uint32)
    return trk, r["trk_offsets"], r["stats"]


def parity_check(b, w, got_trk, got_off, n_events, threads):
    """Compares the GPU's tracklets (input positions) of the first n_events
    of batch b with the oracle run on those events alone."""
    n = min(n_events, b.n_events)
    sample = b.slice_events(0, n)
    want, want_off, _ = oracle_tracklets(sample, w, threads)
    T = w.n_triplets
    k = int(got_off[n * T])
    ok = (np.array_equal(np.asarray(got_trk)[:k], want)
          and np.array_equal(np.asarray(got_off)[: n * T + 1], want_off))
    return {"parity": "bit-exact" if ok else "MISMATCH", "events_checked": n,
            "tracklets_checked": int(k), "against": "CPU oracle (pinned to the reference kernels)"}


def cpu_events_per_s(b, w, seconds, threads, runner=None):
    """A CPU implementation on a bounded sample of b (about `seconds` of CPU
    work): `runner(sample, w)` (the reference's kernels on the host, from
    reference_runner), else the oracle."""
    if runner is None:
        import oracle
        runner = lambda s, w_: oracle.run(s, w_.config(), w_.grid(s.n_events), 4, 256,
                                          threads)["stats"]
    t0 = time.perf_counter()
    probe = b.slice_events(0, min(2, b.n_events))
    runner(probe, w)
    dt = max(time.perf_counter() - t0, 1e-3)
    n = int(max(1, min(b.n_events, probe.n_events * seconds / dt)))
    sample = b.slice_events(0, n)
    t0 = time.perf_counter()
    stats = runner(sample, w)
    dt = time.perf_counter() - t0
    return n / dt, n, dt, stats


# --------------------------------------------------------------------------
# reference arm

# the reference sizes and indexes its pair bitmap (n1 * n2 bits per event and
# layer triplet) in 32-bit counts (PairGeneratorBeamspot.cpp:9-27): event groups
# stay below this many bits, as its own event grouping would keep them
REF_GROUP_BITS = 1 << 31


def reference_groups(b, w):
    """Consecutive event groups of batch b whose pair bitmaps stay within
    REF_GROUP_BITS (at least one event each)."""
    cfg = w.config()
    ln = b.layer_nhits.astype(np.int64)
    bits = np.zeros(b.n_events, dtype=np.int64)
    for t in range(cfg.n_layer_triplets):
        tr = cfg.triplets[t]
        bits += ln[:, tr.layer1 - 1] * ln[:, tr.layer2 - 1]
    groups, first, acc = [], 0, 0
    for e in range(b.n_events):
        if e > first and acc + bits[e] > REF_GROUP_BITS:
            groups.append((first, e - first))
            first, acc = e, 0
        acc += int(bits[e])
    groups.append((first, b.n_events - first))
    return groups


def reference_runner(threads):
    """The reference's own kernels on the host when oracle/_ref builds here
    (run per event group, see REF_GROUP_BITS), else the CPU restatement of its
    algorithm."""
    from oracle import ref
    try:
        if ref.available():
            ref.lib()

            def run_groups(s, w):
                total = None
                for first, count in reference_groups(s, w):
                    g = s.slice_events(first, count) if count != s.n_events else s
                    st = ref.run(g, w.config(), w.grid(g.n_events), 4, n_threads=256,
                                 grid_threads=1, workers=threads)["stats"]
                    total = dict(st) if total is None else {k: total[k] + st[k] for k in st}
                return total
            return "reference", run_groups
    except (OSError, FileNotFoundError, subprocess.CalledProcessError):
        pass
    import oracle
    return "port", lambda s, w: oracle.run(s, w.config(), w.grid(s.n_events), 4, 256,
                                           threads)["stats"]


def run_reference(args, dist):
    from trax_gb300 import gen
    w = workload_at_grid(gen.WORKLOADS[args.workload], args.grid)
    if dist.rank != 0:
        return
    threads = os.cpu_count() or 1
    kind, runner = reference_runner(threads)
    b = gen.generate_batch(w, args.events)
    per_step_s = max(2.0, 150.0 / max(1, args.steps + args.warmup))
    t0 = time.perf_counter()
    probe = b.slice_events(0, min(2, b.n_events))
    runner(probe, w)
    dt = max(time.perf_counter() - t0, 1e-3)
    n = int(max(1, min(b.n_events, probe.n_events * per_step_s / dt)))
    sample = b.slice_events(0, n)
    for _ in range(args.warmup):
        runner(sample, w)
    times = []
    stats = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        stats = runner(sample, w)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    what = ("the reference's OpenCL kernels compiled for the host (oracle/_ref), "
            f"work-groups spread over {threads} threads" if kind == "reference" else
            f"CPU restatement of the reference's algorithm, OpenMP over {threads} threads")
    line = {
        "impl": "reference", "metric": "events/s", "value": round(value, 3), "unit": "events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "events_per_step": n,
                   "grid": f"{w.n_sectors_z}x{w.n_sectors_phi}", "layer_triplets": w.n_triplets,
                   "sample": f"first {n} of the {args.events}-event batch per step"},
        "cpu_baseline": {"value": round(value, 3), "unit": "events/s", "cores": threads,
                         "kind": kind, "sample": f"{n} events per step, {what}"},
        "e2e": {"value": round(value, 3), "unit": "events/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "triplets_per_s": round(stats["tracklets"] * args.steps / total, 1),
        "pairs_per_s": round(stats["pairs"] * args.steps / total, 1),
        "note": ("reference host side (clever, Boost, protobuf 2.4, OpenCL runtime) unbuildable "
                 "here; " + what),
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm

def sized_pipeline(ctx, w, b, caps_per_hit=SIZING_CAPS):
    """A Pipeline whose capacities fit b: a first run at generous per-hit
    capacities (doubled while an output overflows), then one sized from the
    counts it reported."""
    from trax_gb300.ops import Pipeline
    from trax_gb300.runtime import TraxError
    N = b.n_hits
    caps = [c * N + 4096 for c in caps_per_hit]
    counts = None
    for _ in range(4):
        p = Pipeline(ctx, w.config(), w.grid(b.n_events), b.n_events, N, *caps)
        try:
            _, _, counts = p.seed(b)
        except TraxError as exc:
            if exc.status != 5:
                raise
            counts = ctx.counts()
        if counts["status"] == 0:
            break
        caps = [2 * c for c in caps]
        del p
    if counts is None or counts["status"] != 0:
        raise SystemExit(f"device status {counts}")
    need = (counts["n_pairs"], counts["n_candidates"], counts["n_tracklets"])
    caps = [int(1.1 * v) + 4096 for v in need]
    del p
    p = Pipeline(ctx, w.config(), w.grid(b.n_events), b.n_events, N, *caps)
    _, _, counts = p.seed(b)
    if counts["status"] != 0:
        raise SystemExit(f"device status {counts}")
    return p, counts


def per_event_form(ctx, w, b, sample):
    """The plain per-event GPU form: one event per launch sequence, no
    graph, a host synchronisation per event."""
    S = min(sample, b.n_events)
    singles = [b.slice_events(e, 1) for e in range(S)]
    from trax_gb300.ops import Pipeline
    N1 = max(s.n_hits for s in singles) + 1
    pe = Pipeline(ctx, w.config(), w.grid(1), 1, N1,
                  *[c * N1 + 4096 for c in SIZING_CAPS])
    for s in singles[:2]:
        pe.stage(s)
        ctx._check(ctx.lib.trax_run_staged_eager(ctx.h))
    ctx.synchronize()
    t0 = time.perf_counter()
    for s in singles:
        pe.stage(s)
        ctx._check(ctx.lib.trax_run_staged_eager(ctx.h))
        ctx.synchronize()
    rate = S / (time.perf_counter() - t0)
    del pe
    return {"value": round(rate, 2), "unit": "events/s",
            "sample": f"{S} events, one launch sequence each, no graph"}


def kernel_times(ctx, p, reps=20):
    import ctypes as C
    ctx._check(ctx.lib.trax_set_profiling(ctx.h, 1))
    p.run_staged()  # captures the profiled graph
    kt = {}
    for _ in range(reps):
        p.run_staged()
        ms = (C.c_float * 64)()
        names = (C.c_char_p * 64)()
        n = C.c_int()
        ctx._check(ctx.lib.trax_kernel_times(ctx.h, ms, names, 64, C.byref(n)))
        for i in range(n.value):
            kt.setdefault(names[i].decode(), []).append(ms[i])
    ctx._check(ctx.lib.trax_set_profiling(ctx.h, 0))
    return {k: statistics.median(v) for k, v in kt.items()}


def resident_rate(ctx, p, b, steps, warmup, dist, clocks=None):
    """events/s of graph replays on the staged batch, CUDA events on the
    context stream, K steps between barriers."""
    p.stage(b)
    for _ in range(warmup):
        p.run_staged()
    ctx.synchronize()
    dist.barrier()
    if clocks is not None:
        clocks.__enter__()
    ctx.synchronize()
    ctx.timer_record(62)
    for _ in range(steps):
        p.run_staged()
    ctx.timer_record(63)
    ctx.synchronize()
    if clocks is not None:
        clocks.__exit__()
    dist.barrier()
    return aggregate_rate(dist, b.n_events, steps, ctx.timer_elapsed_ms(62, 63))


def pinned_copy(ctx, b):
    """The batch's columns the batched calls upload (x, y, z, layer, event) in
    pinned host memory, the detector and hit ids left out (they are never
    read on that path); returns (batch, buffers to free)."""
    from trax_gb300.gen import EventBatch
    from trax_gb300.runtime import PinnedBuffer
    bufs, cols = [], {}
    for name in ("x", "y", "z", "layer", "event"):
        c = getattr(b, name)
        buf = PinnedBuffer(ctx, c.nbytes, c.dtype)
        buf.array[:] = c
        bufs.append(buf)
        cols[name] = buf.array
    return EventBatch(detector_id=None, hit_id=None, layer_nhits=b.layer_nhits, **cols), bufs


def measure_section(ctx, w, B, args, dist, threads):
    """A further workload: resident value, one-at-a-time e2e, the per-event
    form, and parity of its tracklets against the oracle."""
    from trax_gb300 import gen
    b = gen.generate_batch(w, B, first_event=replica_first_event(dist.rank, B))
    p, counts = sized_pipeline(ctx, w, b)
    from trax_gb300.autotune import tune_walk
    best_walk, _ = tune_walk(ctx, p, b, reps=3)
    steps = max(3, args.steps // 2)
    value, ms_total, events_all = resident_rate(ctx, p, b, steps, args.warmup, dist)
    pb, bufs = pinned_copy(ctx, b)
    p.seed(pb, input_indices=True, copy=False)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        p.seed(pb, input_indices=True, copy=False)
    sync_s = dist.max(time.perf_counter() - t0)
    for x in bufs:
        x.free()
    trk, off, _ = p.seed(b, input_indices=True)
    par = parity_check(b, w, trk, off, B if B <= 128 else args.parity_events, threads)
    del p
    pe = per_event_form(ctx, w, b, args.per_event_sample)
    return {"workload": w.name, "events_per_step": B, "hits_per_step": b.n_hits,
            "grid": f"{w.n_sectors_z}x{w.n_sectors_phi}", "value": round(value, 2),
            "unit": "events/s", "ms_per_step": round(ms_total / steps, 4),
            "e2e_sync": {"value": round(events_all * steps / sync_s, 2),
                         "form": "trax_seed_batch, one batch at a time (pinned H2D + D2H)"},
            "triplets_per_s": round(counts["n_tracklets"] * dist.world * steps /
                                    (ms_total / 1000), 1),
            "per_event_form": pe,
            "batched_over_per_event": round(value / dist.world / pe["value"], 2),
            "walk": list(best_walk), **par}


def run_autotune(args, ctx):
    """Config 4: pile-up-200 events, grid sweep {8..320} x {16..192} with the
    walk tuned per grid, the plain per-event form at the best grid."""
    from trax_gb300 import gen
    from trax_gb300.autotune import sweep_grids, density_class, GRID_Z, GRID_PHI, MAX_CELLS
    w = gen.WORKLOADS["pileup200"]
    b = gen.generate_batch(w, args.autotune_events)
    grids = [(z, ph) for z in GRID_Z for ph in GRID_PHI if (z + 1) * (ph + 1) <= MAX_CELLS]
    grids.append((12, 32))
    t0 = time.perf_counter()
    rows = sweep_grids(ctx, w, b, grids=grids, reps=3)
    best = rows[0]
    wk = gen.Workload(w.name, w.config_id, w.n_layers, w.noise, w.pt_range,
                      best["n_sectors_z"], best["n_sectors_phi"], w.n_triplets,
                      pileup_mean=w.pileup_mean)
    pe = per_event_form(ctx, wk, b, 16)
    return {"workload": w.name, "events": b.n_events,
            "hits_per_event": round(b.n_hits / b.n_events, 1),
            "class": density_class(b.n_hits / b.n_events), "best": best,
            "default_12x32": next((r for r in rows if r.get("grid") == "12x32"), None),
            "per_event_form_at_best": pe,
            "batched_over_per_event_at_best": round(best["events_per_s"] / pe["value"], 2),
            "headline_grid": "x".join(map(str, TUNED_GRID["pileup200"])),
            "headline_grid_is_best": best["grid"] == "x".join(map(str, TUNED_GRID["pileup200"])),
            # the headline grid's own sweep rate against the best one (grids within
            # a percent or two trade places between sweeps)
            "headline_over_best": next((round(r["events_per_s"] / best["events_per_s"], 4)
                                        for r in rows if r.get("grid") ==
                                        "x".join(map(str, TUNED_GRID["pileup200"]))), None),
            "sweep_s": round(time.perf_counter() - t0, 1),
            "sweep": [{k: r[k] for k in ("grid", "events_per_s", "walk") if k in r}
                      for r in rows]}


def run_serving(args):
    """Poisson streams of pile-up ~ U{0..200} events through the
    continuous-batching server; p50/p99 arrival-to-result latency."""
    from trax_gb300 import gen
    from trax_gb300.serve import Server, poisson_arrivals
    w = workload_at_grid(gen.WORKLOADS["stream-pileup-u200"], args.serve_grid)
    tuning = None
    if args.serve_walk:
        tuning = [int(v) for v in args.serve_walk.split(",")]
    elif args.serve_grid == "tuned" and w.name in TUNED_WALK:
        tuning = list(TUNED_WALK[w.name])
    pool = [gen.generate_batch(w, 1, first_event=i) for i in range(args.serve_pool)]
    hits = np.array([e.n_hits for e in pool])
    out = {"workload": w.name, "grid": f"{w.n_sectors_z}x{w.n_sectors_phi}",
           "pool_events": len(pool), "hits_per_event_mean": round(float(hits.mean()), 1),
           "hits_per_event_max": int(hits.max()), "slots": 3, "max_batch_events": 256,
           "rates": []}
    out["tuning"] = tuning
    with Server(w.config(), w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=3,
                max_batch_events=256, max_event_hits=int(hits.max()) + 1,
                memory_budget_bytes=24 << 30, keep_results=False, tuning=tuning) as srv:
        # warm-up: every slot captures its graph
        srv.replay(pool, np.arange(len(pool)) % len(pool),
                   np.full(len(pool), srv.now_ns(), dtype=np.uint64))
        srv.drain()
        for rate in [float(r) for r in args.serve_rates.split(",") if r]:
            srv.reset_stats()
            n = max(1, int(rate * args.serve_seconds))
            order = np.random.default_rng(int(rate)).integers(0, len(pool), n)
            arr = poisson_arrivals(n, rate, srv.now_ns() + 5_000_000, seed=int(rate))
            srv.replay(pool, order, arr)
            srv.drain(timeout_ms=600_000)
            st = srv.stats()
            out["rates"].append({
                "offered_events_per_s": rate, "events": st["events"],
                "sustained_events_per_s": round(st["sustained_events_per_s"], 1),
                "p50_ms": round(st["p50_ns"] / 1e6, 3), "p99_ms": round(st["p99_ns"] / 1e6, 3),
                "max_ms": round(st["max_ns"] / 1e6, 3),
                "mean_batch_events": round(st["batched_events"] / max(1, st["batches"]), 2),
                "splits": st["splits"], "errors": st["errors"]})
    return out


def run_ours(args, dist):
    from trax_gb300 import Context, gen
    from trax_gb300.autotune import tune_walk

    threads = os.cpu_count() or 1
    w = workload_at_grid(gen.WORKLOADS[args.workload], args.grid)
    ctx = Context(dist.local)
    B = args.events
    b = gen.generate_batch(w, B, first_event=replica_first_event(dist.rank, B))
    N = b.n_hits
    if args.walk:
        # a given walk runs from the sizing chains on, so that every chain a
        # profiler sees is the measured one
        best_walk = tuple(int(v) for v in args.walk.split(","))
        ctx.set_tuning(*best_walk)
    p, counts = sized_pipeline(ctx, w, b)

    # ---- result-neutral walk tuning on the resident batch ------------------
    if args.walk:
        walk_ms = {}
    else:
        best_walk, walk_ms = tune_walk(ctx, p, b, reps=3)
    tuning = {"run_walk": best_walk[0], "index_min": best_walk[1], "pair_record": best_walk[2],
              "candidates_ms": {"/".join(map(str, k)): round(v, 4) for k, v in walk_ms.items()}}

    # ---- device-resident value: graph replay on staged inputs -------------
    clk = ClockSampler(dist.local)
    value, ms_total, events_all = resident_rate(ctx, p, b, args.steps, args.warmup, dist, clk)
    launches = int(ctx.lib.trax_kernel_launches(ctx.h))
    counts = ctx.counts()
    if counts["status"] != 0:
        raise SystemExit(f"device status after timed run {counts}")
    if args.only_resident:
        kms = {k: round(v, 4) for k, v in kernel_times(ctx, p, reps=5).items()} \
            if os.environ.get("TRAX_BENCH_KERNELS") else None
        if dist.rank == 0:
            print(json.dumps({"metric": "events/s", "value": round(value, 2), "unit": "events/s",
                              "kernels_ms": kms,
                              "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": round(ms_total / args.steps, 4),
                              "config": {"workload": args.workload, "events_per_step": B,
                                         "grid": f"{w.n_sectors_z}x{w.n_sectors_phi}",
                                         "walk": list(best_walk)},
                              "note": "resident graph replays only (--only-resident)"}), flush=True)
        ctx.close()
        return

    # ---- per-kernel times (separate profiled run) and roofline ------------
    kernel_ms = kernel_times(ctx, p)
    top = max(kernel_ms, key=kernel_ms.get)
    peak, peak_src = hbm_peak()
    kernels = {}
    for k, v in kernel_ms.items():
        alg = algorithmic_bytes(k, b, w, counts)
        e = {"ms": round(v, 4)}
        if alg and v > 0:
            e["gbs"] = round(alg / (v / 1000) / 1e9, 1)
            e["hbm_frac"] = round(alg / (v / 1000) / 1e9 / peak, 4)
        kernels[k] = e
    if "grid_build" in kernel_ms:
        act = grid_build_actual_bytes(b, w)
        g = kernels["grid_build"]
        g["reference_equivalent_bytes"] = algorithmic_bytes("grid_build", b, w, counts)
        g["actual_column_bytes"] = act
        g["hbm_frac_actual_columns"] = round(act / (kernel_ms["grid_build"] / 1000) / 1e9 / peak, 4)
    pair_ms = sum(kernel_ms.get(k, 0) for k in ("pair_gen", "pair_scan", "pair_store"))
    if pair_ms > 0:
        pb = algorithmic_bytes("pair_gen", b, w, counts)
        kernels["pair_stage_total"] = {"ms": round(pair_ms, 4),
                                       "hbm_frac": round(pb / (pair_ms / 1000) / 1e9 / peak, 4)}
    alg = algorithmic_bytes(top, b, w, counts)
    roofline = None
    if alg is not None:
        achieved = alg / (kernel_ms[top] / 1000.0) / 1e9
        roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2),
                    "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5),
                    "traffic": profile_entry(args.workload, top),
                    "algorithmic_bytes": int(alg), "launch_ms": round(kernel_ms[top], 4),
                    "peak_source": peak_src,
                    "sm_issue_active": (profile_entry(args.workload, "_sm_issue_active") or {}).get(top),
                    "timing": "median of 20 profiled graph replays, CUDA events between kernels "
                              "(the events add about 3 % to each kernel)",
                    "note": "not DRAM-bound: the hits of a layer stay in L1/L2; the kernel is "
                            "bound by instruction issue and load latency (sm_issue_active from ncu)"}

    # ---- e2e through the streaming API with pinned host buffers -----------
    pinned_batch, pinned = pinned_copy(ctx, b)
    for _ in range(args.warmup):
        p.seed(pinned_batch, copy=False)
    dist.barrier()
    ctx.synchronize()
    t0 = time.perf_counter()
    trk = None
    for _ in range(args.steps):
        trk, off, c2 = p.seed(pinned_batch, copy=False)
    sync_s = dist.max(time.perf_counter() - t0)

    def stream(k):
        tickets = []
        res = None
        for i in range(k):
            tickets.append(p.submit(pinned_batch))
            if i >= 1:
                res = p.wait(tickets[i - 1], copy=False)
        return p.wait(tickets[-1], copy=False), res
    stream(args.warmup)
    dist.barrier()
    ctx.synchronize()
    t0 = time.perf_counter()
    (strk, soff, sc2), _ = stream(args.steps)
    e2e_s = dist.max(time.perf_counter() - t0)
    if sc2["n_tracklets"] != c2["n_tracklets"] or not np.array_equal(strk[0], trk[0]):
        raise SystemExit("streaming result differs from the synchronous one")
    # the batched calls upload x, y, z, layer and event (the detector and hit
    # ids are not read on that path) and the segment starts and counts
    h2d = sum(c.nbytes for c in (b.x, b.y, b.z, b.layer, b.event)) + 2 * b.layer_nhits.nbytes + 8
    d2h = int(sum(t.nbytes for t in trk) + off.nbytes + 72)
    e2e = {"value": round(events_all * args.steps / e2e_s, 2), "unit": "events/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": d2h,
           "ms_per_step": round(1000 * e2e_s / args.steps, 3),
           "form": "trax_submit_batch / trax_wait_batch, 2 batches in flight",
           "sync": {"value": round(events_all * args.steps / sync_s, 2),
                    "ms_per_step": round(1000 * sync_s / args.steps, 3),
                    "form": "trax_seed_batch, one batch at a time"}}
    for x in pinned:
        x.free()

    # ---- parity of the timed batch against the oracle ----------------------
    trk_in, off_in, _ = p.seed(b, input_indices=True)
    parity = parity_check(b, w, trk_in, off_in, args.parity_events, threads)
    if parity["parity"] != "bit-exact":
        print(json.dumps({"error": "GPU tracklets differ from the oracle", **parity}),
              file=sys.stderr)
        raise SystemExit(3)
    del p

    # ---- plain per-event GPU form (no graph, one event per sequence) -----
    pe = per_event_form(ctx, w, b, args.per_event_sample)

    # ---- PrefixSum micro-benchmark: 1 Mi uint32, the reference's own
    # prefix-sum benchmark shape (src/trax_test/trax_test.cpp:436-479)
    n_scan = 1024 * 1024
    d_scan = ctx.upload(np.ones(n_scan, np.uint32))
    for _ in range(5):
        ctx.prefix_sum(d_scan, d_scan, n_scan)
    ctx.synchronize()
    reps = 100
    ctx.timer_record(60)
    for _ in range(reps):
        ctx.prefix_sum(d_scan, d_scan, n_scan)
    ctx.timer_record(61)
    scan_ms = ctx.timer_elapsed_ms(60, 61) / reps
    prefix_sum = {"n": n_scan, "ms": round(scan_ms, 5),
                  "gbs": round(8 * n_scan / (scan_ms / 1000) / 1e9, 1),
                  "note": "in place, 4 B read + 4 B written per element"}

    # ---- further workloads (configs 3 and 2) -------------------------------
    sections = {}
    if not args.no_sections:
        for name, ev in SECTIONS:
            if name == args.workload:
                continue
            sections[name] = measure_section(ctx, gen.WORKLOADS[name], ev, args, dist, threads)
            if sections[name]["parity"] != "bit-exact":
                print(json.dumps({"error": "GPU tracklets differ from the oracle",
                                  "section": name}), file=sys.stderr)
                raise SystemExit(3)

    # ---- autotuned sweep (config 4) --------------------------------------
    autotune = None
    if not args.no_autotune and dist.world == 1:
        autotune = run_autotune(args, ctx)

    # ---- streaming serving load (config 5) --------------------------------
    serving = None
    if args.serve_rates and dist.world == 1:
        serving = run_serving(args)

    # ---- CPU baseline (rank 0, N=1 only) ----------------------------------
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        kind, runner = reference_runner(threads)
        v, n, dt, _ = cpu_events_per_s(b, w, args.cpu_seconds, threads, runner)
        v1, n1, dt1, _ = cpu_events_per_s(b, w, max(2.0, args.cpu_seconds / 2), 1,
                                          reference_runner(1)[1])
        what = ("the reference's OpenCL kernels compiled for the host (oracle/_ref), "
                "work-groups spread over the threads" if kind == "reference"
                else "OpenMP oracle")
        cpu = {"value": round(v, 3), "unit": "events/s", "cores": threads, "kind": kind,
               "sample": f"first {n} events of the batch, {dt:.1f} s, {what}",
               "one_thread": {"value": round(v1, 3), "cores": 1,
                              "sample": f"first {n1} events, {dt1:.1f} s"}}
        if kind == "reference":
            vp, np_, dtp, _ = cpu_events_per_s(b, w, max(2.0, args.cpu_seconds / 2), threads)
            cpu["port"] = {"value": round(vp, 3), "cores": threads,
                           "sample": f"first {np_} events, {dtp:.1f} s, OpenMP oracle"}

    clocks = clk.summary()
    if dist.rank == 0:
        mb_resident = (N * (28 + 36) + counts["n_pairs"] * 8 + counts["n_candidates"] * 8) / 1e6
        line = {
            "metric": "events/s", "value": round(value, 2), "unit": "events/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_total / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "events_per_step": B, "hits_per_step": N,
                       "hits_per_event": round(N / B, 1),
                       "layers": w.n_layers, "layer_triplets": w.n_triplets,
                       "grid": f"{w.n_sectors_z}x{w.n_sectors_phi}",
                       "grid_source": ("autotuner (sweep on pile-up-200 events; see 'autotune')"
                                       if args.grid == "tuned" and args.workload in TUNED_GRID
                                       else "workload"),
                       "form": "batched: one CUDA graph per step",
                       "l2": f"inputs larger than L2 ({mb_resident:.0f} MB touched per step)",
                       "parallelism": f"replicas x{dist.world}"},
            "e2e": e2e,
            "pairs_per_s": round(counts["n_pairs"] * dist.world * args.steps / (ms_total / 1000), 1),
            "triplets_per_s": round(counts["n_tracklets"] * dist.world * args.steps / (ms_total / 1000), 1),
            "per_event_form": pe,
            "batched_over_per_event": round(value / dist.world / pe["value"], 2),
            "parity": parity["parity"], "parity_detail": parity,
            "roofline": roofline,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "prefix_sum_1mi": prefix_sum,
            "sections": sections,
            "serving": serving,
            "tuning": tuning,
            "autotune": autotune,
            "clocks": clocks,
            "gpu_launches": launches * args.steps,
            "counts_per_step": {k: counts[k] for k in ("n_hits", "n_pairs", "pair_slots",
                                                        "n_candidates", "cand_slots",
                                                        "cand_truncated", "n_tracklets")},
        }
        print(json.dumps(line), flush=True)
    ctx.close()


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    args = parse(argv)
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        return launch_replicas(args.gpus, argv)
    if "WORLD_SIZE" in os.environ and int(os.environ["WORLD_SIZE"]) != args.gpus:
        print(f"--gpus {args.gpus} disagrees with WORLD_SIZE={os.environ['WORLD_SIZE']}",
              file=sys.stderr)
        return 2
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
