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

    def set_tuning(self, run_walk, index_min, pair_record):
        self.tuning = (run_walk, index_min, pair_record)
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


def test_tune_walk_times_every_walk_then_the_pair_kernels_at_the_best(monkeypatch):
    table = {(96, 32, 3): 2.0, (96, 32, 2): 1.5, (96, 32, 1): 3.0, (96, 32, 0): 4.0}
    ctx, p, best, timings = _tune(monkeypatch, table)
    assert p.staged == "b"
    walks = [(*c, 3) for c in autotune.WALK_CANDIDATES]
    assert ctx.history[:len(walks)] == walks
    # the other pair kernels run only at the best walk, in the documented order
    assert ctx.history[len(walks):len(walks) + 3] == [(96, 32, 2), (96, 32, 1), (96, 32, 0)]
    assert best == (96, 32, 2)
    assert ctx.tuning == best  # installed last
    assert len(timings) == len(walks) + 3


def test_tune_walk_keeps_the_split_pair_stage_when_it_is_fastest(monkeypatch):
    table = {(0, 16, 3): 1.0}
    ctx, _, best, _ = _tune(monkeypatch, table)
    assert best == (0, 16, 3)
    assert ctx.tuning == (0, 16, 3)
    assert ctx.history[-4:-1] == [(0, 16, 2), (0, 16, 1), (0, 16, 0)]


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
