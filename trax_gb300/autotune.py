"""Autotuner for the seeding pipeline.

Two kinds of knob, tuned differently:
- how the candidate kernels visit a window and how they are launched
  (trax_set_tuning: walk runs of cells or search a per-cell z index; which
  pair kernels run; how many blocks per SM the candidate kernels keep
  resident -- the launch shape the reference sweeps as its work-group size).
  Results never depend on them, so tune_walk() simply times the candidates on
  the resident batch and keeps the fastest.
- the grid granularity (z bins x phi bins).  It changes which candidates the
  reference visits first and therefore its truncation, so a tuned grid is a
  different (but equally reference-defined) configuration; sweep_grids()
  reports events/s per grid and hit-density class, and parity at a chosen
  grid is checked against the oracle run at that grid.
"""
from __future__ import annotations

import math

import numpy as np

from . import gen
from .ops import Pipeline
from .runtime import Context

WALK_CANDIDATES = ((1 << 30, 256), (96, 256), (96, 32), (48, 16), (24, 8), (0, 16), (0, 0))
# resident blocks per SM of the candidate kernels (0: as many as fit)
BLOCK_CAPS = (4, 3, 2)
GRID_Z = (8, 16, 32, 64, 128, 256, 320)
GRID_PHI = (16, 32, 64, 128, 192)
# cells per layer the library accepts ((n_sectors_z + 1) * (n_sectors_phi + 1))
MAX_CELLS = 65536
TIMER_A, TIMER_B = 56, 57


def time_staged(ctx: Context, p: Pipeline, reps: int) -> float:
    """Median ms of `reps` graph replays on the staged batch."""
    p.run_staged()  # (re)captures the graph
    ctx.synchronize()
    times = []
    for _ in range(reps):
        ctx.timer_record(TIMER_A)
        p.run_staged()
        ctx.timer_record(TIMER_B)
        times.append(ctx.timer_elapsed_ms(TIMER_A, TIMER_B))
    return float(np.median(times))


def tune_walk(ctx: Context, p: Pipeline, batch: gen.EventBatch, reps=5,
              candidates=WALK_CANDIDATES, block_caps=BLOCK_CAPS):
    """Stages `batch`, times each (run_walk, index_min) with the split
    one-outer-hit-per-lane pair stage, then the best of them with the other
    pair kernels (one outer hit per lane with look-back, the warp sweep
    replaying its ballots, the warp sweep twice), then the best of those with
    fewer resident blocks per SM, and installs the fastest
    (run_walk, index_min, pair_record, blocks_per_sm)."""
    p.stage(batch)
    timings = {}
    for cand in candidates:
        ctx.set_tuning(*cand, 3, 0)
        timings[(*cand, 3, 0)] = time_staged(ctx, p, reps)
    best = min(timings, key=timings.get)
    for rec in (2, 4, 1, 0):
        ctx.set_tuning(best[0], best[1], rec, 0)
        timings[(best[0], best[1], rec, 0)] = time_staged(ctx, p, reps)
    best = min(timings, key=timings.get)
    for cap in block_caps:
        t = (best[0], best[1], best[2], cap)
        ctx.set_tuning(*t)
        timings[t] = time_staged(ctx, p, reps)
    best = min(timings, key=timings.get)
    ctx.set_tuning(*best)
    return best, timings


def tuning_for(table, hits_per_event: float):
    """The tuning `table` (density class -> tuning tuple, as autotune()
    reports under "walk") holds for a batch of this density, or None."""
    if not table:
        return None
    t = table.get(density_class(hits_per_event))
    return tuple(t) if t is not None else None


def density_class(hits_per_event: float) -> str:
    if hits_per_event < 5_000:
        return "sparse(<5k hits/event)"
    if hits_per_event < 20_000:
        return "medium(5k-20k)"
    return "dense(>=20k)"


def sweep_grids(ctx: Context, w: gen.Workload, batch: gen.EventBatch, grids=None, reps=3,
                caps=(80, 80, 8)):
    """events/s of the batched pipeline at each grid, with the walk tuned per
    grid.  Returns a list of dicts sorted by events/s (best first)."""
    grids = grids or [(z, p) for z in GRID_Z for p in GRID_PHI if (z + 1) * (p + 1) <= MAX_CELLS]
    N = batch.n_hits
    rows = []
    for nz, nphi in grids:
        wk = gen.Workload(w.name, w.config_id, w.n_layers, w.noise, w.pt_range, nz, nphi,
                          w.n_triplets, tracks=w.tracks, pileup_mean=w.pileup_mean,
                          pileup_uniform=w.pileup_uniform)
        p = Pipeline(ctx, wk.config(), wk.grid(batch.n_events), batch.n_events, N,
                     caps[0] * N, caps[1] * N, caps[2] * N)
        _, _, counts = p.seed(batch)
        if counts["status"] != 0:
            rows.append({"grid": f"{nz}x{nphi}", "status": counts["status"]})
            continue
        best, timings = tune_walk(ctx, p, batch, reps=reps)
        ms = timings[best]
        rows.append({"grid": f"{nz}x{nphi}", "n_sectors_z": nz, "n_sectors_phi": nphi,
                     "walk": list(best), "ms": round(ms, 4),
                     "events_per_s": round(batch.n_events / (ms / 1000.0), 1),
                     "tracklets": counts["n_tracklets"], "pairs": counts["n_pairs"]})
        del p
    ok = [r for r in rows if "ms" in r]
    ok.sort(key=lambda r: -r["events_per_s"])
    return ok + [r for r in rows if "ms" not in r]


def autotune(ctx: Context, w: gen.Workload, batches, grids=None, reps=3):
    """Best grid and tuning per hit-density class over the given sample
    batches.  The "tuning" of each class is what Pipeline(tuning_by_class=)
    and Server(tuning=) apply."""
    out = {}
    for b in batches:
        cls = density_class(b.n_hits / max(1, b.n_events))
        rows = sweep_grids(ctx, w, b, grids=grids, reps=reps)
        out[cls] = {"hits_per_event": round(b.n_hits / max(1, b.n_events), 1),
                    "events": b.n_events, "best": rows[0] if rows else None, "sweep": rows,
                    "tuning": rows[0]["walk"] if rows else None}
    return out
