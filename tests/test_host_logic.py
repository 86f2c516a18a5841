"""Host-side logic that needs no GPU: the autotuner's candidate order and
selection (timed through a fake context), the hit-density classes, and the
Poisson arrival stream the serving measurement replays."""
import numpy as np

from trax_gb300 import autotune
from trax_gb300.serve import poisson_arrivals


class _FakeCtx:
    def __init__(self):
        self.tuning = None
        self.history = []

    def set_tuning(self, run_walk, index_min, pair_record, blocks_per_sm=0):
        self.tuning = (run_walk, index_min, pair_record, blocks_per_sm)
        self.history.append(self.tuning)


class _FakePipeline:
    def __init__(self):
        self.staged = None

    def stage(self, batch):
        self.staged = batch


def _tune(monkeypatch, table, default=10.0):
    ctx, p = _FakeCtx(), _FakePipeline()
    monkeypatch.setattr(autotune, "time_staged",
                        lambda c, pipe, reps: table.get(c.tuning, default))
    best, timings = autotune.tune_walk(ctx, p, batch="b", reps=1)
    return ctx, p, best, timings


def test_tune_walk_times_every_walk_then_the_pair_kernels_then_the_launch_shape(monkeypatch):
    table = {(96, 32, 3, 0): 2.0, (96, 32, 2, 0): 1.5, (96, 32, 1, 0): 3.0,
             (96, 32, 0, 0): 4.0, (96, 32, 2, 3): 1.2}
    ctx, p, best, timings = _tune(monkeypatch, table)
    assert p.staged == "b"
    walks = [(*c, 3, 0) for c in autotune.WALK_CANDIDATES]
    assert ctx.history[:len(walks)] == walks
    # the other pair kernels run only at the best walk, in the documented order
    n = len(walks)
    assert ctx.history[n:n + 4] == [(96, 32, 2, 0), (96, 32, 4, 0), (96, 32, 1, 0),
                                    (96, 32, 0, 0)]
    # then fewer resident blocks per SM at the best of those
    assert ctx.history[n + 4:n + 4 + len(autotune.BLOCK_CAPS)] == \
        [(96, 32, 2, c) for c in autotune.BLOCK_CAPS]
    assert best == (96, 32, 2, 3)
    assert ctx.tuning == best  # installed last
    assert len(timings) == n + 4 + len(autotune.BLOCK_CAPS)


def test_tune_walk_keeps_the_split_pair_stage_when_it_is_fastest(monkeypatch):
    table = {(0, 16, 3, 0): 1.0}
    ctx, _, best, _ = _tune(monkeypatch, table)
    assert best == (0, 16, 3, 0)
    assert ctx.tuning == (0, 16, 3, 0)
    caps = len(autotune.BLOCK_CAPS)
    assert ctx.history[-5 - caps:-1 - caps] == [(0, 16, 2, 0), (0, 16, 4, 0), (0, 16, 1, 0),
                                                (0, 16, 0, 0)]


def test_tuning_for_picks_the_batch_class():
    table = {"dense(>=20k)": [1 << 30, 256, 2, 3], "sparse(<5k hits/event)": [48, 16, 3, 0]}
    assert autotune.tuning_for(table, 26_000.0) == (1 << 30, 256, 2, 3)
    assert autotune.tuning_for(table, 3_000.0) == (48, 16, 3, 0)
    assert autotune.tuning_for(table, 10_000.0) is None
    assert autotune.tuning_for(None, 10_000.0) is None


def test_density_classes():
    assert autotune.density_class(0) == "sparse(<5k hits/event)"
    assert autotune.density_class(4_999.9) == "sparse(<5k hits/event)"
    assert autotune.density_class(5_000) == "medium(5k-20k)"
    assert autotune.density_class(19_999) == "medium(5k-20k)"
    assert autotune.density_class(20_000) == "dense(>=20k)"


def test_poisson_arrivals_are_a_seeded_increasing_stream_at_the_rate():
    start = 1_000_000_000
    a = poisson_arrivals(20_000, 5_000.0, start, seed=7)
    assert a.dtype == np.uint64 and len(a) == 20_000
    assert (a > start).all()
    assert (np.diff(a.astype(np.int64)) >= 0).all()
    assert np.array_equal(a, poisson_arrivals(20_000, 5_000.0, start, seed=7))
    assert not np.array_equal(a, poisson_arrivals(20_000, 5_000.0, start, seed=8))
    mean_gap_s = (int(a[-1]) - start) / 1e9 / len(a)
    assert abs(mean_gap_s * 5_000.0 - 1.0) < 0.03


def test_batch_struct_passes_null_id_columns():
    """The batched calls never read the detector and hit ids: a batch that
    leaves them out (None) reaches the C-ABI with null pointers there and
    the five columns it uploads intact."""
    import dataclasses
    from trax_gb300 import gen
    from trax_gb300 import _abi as A
    from trax_gb300.ops import _col_ptrs, _host_cols
    b = gen.generate_batch(gen.WORKLOADS["multimuon-1000trk"], 2)
    nb = dataclasses.replace(b, detector_id=None, hit_id=None)
    cols = _host_cols(nb)
    assert cols[4] is None and cols[5] is None
    ln = np.ascontiguousarray(nb.layer_nhits.reshape(-1), dtype=np.uint32)
    s = A.TraxEventBatch(nb.n_events, nb.n_layers, nb.n_hits, *_col_ptrs(cols), ln.ctypes.data)
    assert s.detector_id is None and s.hit_id is None
    for name, c in zip(("x", "y", "z", "layer", "event"), (cols[0], cols[1], cols[2], cols[3], cols[6])):
        assert getattr(s, name) == c.ctypes.data
    assert s.n_hits == b.n_hits and s.n_events == 2


def test_grid_sweep_includes_the_headline_grid():
    """The bench's headline grid for pile-up 200 lies inside the autotuner's
    sweep, within the cell limit."""
    import bench
    z, p = bench.TUNED_GRID["pileup200"]
    assert z in autotune.GRID_Z and p in autotune.GRID_PHI
    assert (z + 1) * (p + 1) <= autotune.MAX_CELLS
