"""Autotuner: the walk knob is result-neutral and the grid sweep's chosen
grid gives oracle-exact tracklets at that grid."""
import numpy as np
import pytest

import oracle
from trax_gb300 import gen
from trax_gb300.autotune import sweep_grids, tune_walk
from trax_gb300.ops import Pipeline

pytestmark = pytest.mark.gpu


def test_tune_walk_installs_a_candidate(gpu_ctx):
    w = gen.WORKLOADS["pileup50-batch100"]
    b = gen.generate_batch(w, 4)
    p = Pipeline(gpu_ctx, w.config(), w.grid(4), 4, b.n_hits, 60 * b.n_hits, 60 * b.n_hits,
                 8 * b.n_hits)
    try:
        best, timings = tune_walk(gpu_ctx, p, b, reps=2)
        assert gpu_ctx.get_tuning() == tuple(best)
        assert all(t > 0 for t in timings.values())
        trk, _, counts = p.seed(b)
        ref = oracle.canonical(oracle.run(b, w.config(), w.grid(4), 4, n_threads=1))
        assert np.array_equal(trk, ref["tracklets"])
    finally:
        gpu_ctx.set_tuning(48, 16)


def test_grid_sweep_best_is_oracle_exact(gpu_ctx):
    base = gen.WORKLOADS["pileup50-batch100"]
    b = gen.generate_batch(base, 2)
    rows = sweep_grids(gpu_ctx, base, b, grids=[(12, 32), (32, 64), (64, 128)], reps=2)
    best = rows[0]
    assert best["events_per_s"] > 0
    wk = gen.Workload(base.name, base.config_id, base.n_layers, base.noise, base.pt_range,
                      best["n_sectors_z"], best["n_sectors_phi"], base.n_triplets,
                      pileup_mean=base.pileup_mean)
    p = Pipeline(gpu_ctx, wk.config(), wk.grid(2), 2, b.n_hits, 80 * b.n_hits, 80 * b.n_hits,
                 8 * b.n_hits)
    trk, off, counts = p.seed(b)
    r = oracle.run(b, wk.config(), wk.grid(2), 4, n_threads=1)
    assert np.array_equal(trk, oracle.canonical(r)["tracklets"])
    assert np.array_equal(off, r["trk_offsets"])
    gpu_ctx.set_tuning(48, 16)


def test_pipeline_and_server_apply_the_class_tuning(gpu_ctx):
    """A per-class tuning table: the pipeline installs the batch's class
    tuning (dense pile-up here) before running it, the server installs the
    given tuning on its slots; neither changes a result."""
    from trax_gb300.autotune import density_class
    from trax_gb300.serve import Server
    w = gen.WORKLOADS["pileup200"]
    b = gen.generate_batch(w, 2)
    cls = density_class(b.n_hits / b.n_events)
    table = {cls: [1 << 30, 256, 2, 3], "sparse(<5k hits/event)": [48, 16, 3, 0]}
    N = b.n_hits
    p = Pipeline(gpu_ctx, w.config(), w.grid(2), 2, N, 48 * N, 96 * N, 8 * N,
                 tuning_by_class=table)
    trk, off, counts = p.seed(b)
    assert gpu_ctx.get_tuning() == (1 << 30, 256, 2, 3)
    ref = oracle.run(b, w.config(), w.grid(2), 4, n_threads=1, omp_threads=8)
    assert np.array_equal(trk, oracle.canonical(ref)["tracklets"])
    gpu_ctx.set_tuning(48, 16)
    one = b.slice_events(0, 1)
    with Server(w.config(), w.n_layers, w.n_sectors_z, w.n_sectors_phi, slots=1,
                max_batch_events=2, memory_budget_bytes=4 << 30,
                tuning=(1 << 30, 256, 2, 3)) as srv:
        t = srv.submit(one, srv.now_ns())
        r = srv.poll(timeout_ms=20_000)
    assert r is not None and r["status"] == 0 and r["ticket"] == t
    r1 = oracle.run(one, w.config(), w.grid(1), 4, n_threads=1, omp_threads=8)
    so = r1["sorted_orig"]
    want = np.stack([so[r1["trk_h1"]], so[r1["trk_h2"]], so[r1["trk_h3"]]], axis=1)
    assert np.array_equal(r["tracklets"], want)
