"""TripletConnectivity on the GPU through the C-ABI: the reference's known
answers, random tables and real tracklets against the oracle."""
import numpy as np
import pytest

import oracle
from connectivity_cases import (FOUR_LAYER, FOUR_LAYER_EXPECT, FOUR_LAYER_TIGHT,
                                FOUR_LAYER_TIGHT_EXPECT, SIMPLE_BACKWARD, SIMPLE_FORWARD)
from trax_gb300 import gen
from trax_gb300.ops import Pipeline, TrackletCollection, TripletConnectivity

pytestmark = pytest.mark.gpu


def _gpu_chain(ctx, layers, tight=False, backwards=False):
    cols = [TrackletCollection.from_host(ctx, np.array(l, np.uint32)) for l in layers]
    op = TripletConnectivity(ctx)
    for base, follow in zip(cols[:-1], cols[1:]):
        op.run(base, follow, iterate_backwards=backwards, tight_packing=tight)
    ctx.synchronize()
    return cols[-1].get_connectivity().tolist()


def test_reference_known_answers(gpu_ctx):
    assert _gpu_chain(gpu_ctx, [SIMPLE_FORWARD["base"], SIMPLE_FORWARD["following"]]) == \
        SIMPLE_FORWARD["expect_following"]
    assert _gpu_chain(gpu_ctx, [SIMPLE_BACKWARD["base"], SIMPLE_BACKWARD["following"]],
                      backwards=True) == SIMPLE_BACKWARD["expect_following"]
    assert _gpu_chain(gpu_ctx, FOUR_LAYER) == FOUR_LAYER_EXPECT
    assert _gpu_chain(gpu_ctx, FOUR_LAYER_TIGHT, tight=True) == FOUR_LAYER_TIGHT_EXPECT


@pytest.mark.parametrize("tight,backwards", [(False, False), (False, True), (True, False)])
def test_random_tables_match_oracle(gpu_ctx, tight, backwards):
    rng = np.random.default_rng(7 + 2 * tight + backwards)
    base = rng.integers(0, 3000, (20000, 3)).astype(np.uint32)
    follow = rng.integers(0, 3000, (15000, 3)).astype(np.uint32)
    if tight:  # make some two-hit overlaps
        follow[:5000, :2] = base[:5000, 1:]
    bcon = rng.integers(0, 5, len(base)).astype(np.uint32)
    fcon = rng.integers(0, 5, len(follow)).astype(np.uint32)
    b = TrackletCollection.from_host(gpu_ctx, base, bcon)
    f = TrackletCollection.from_host(gpu_ctx, follow, fcon)
    TripletConnectivity(gpu_ctx).run(b, f, iterate_backwards=backwards, tight_packing=tight)
    gpu_ctx.synchronize()
    want = oracle.connectivity(base, bcon, follow, fcon, backwards, tight)
    assert np.array_equal(f.get_connectivity(), want)


def test_real_tracklets_tight(gpu_ctx):
    """Triplets of (1,2,3) chained with triplets of (2,3,4) sharing two hits."""
    w = gen.WORKLOADS["multimuon-1000trk"]
    b = gen.generate_batch(w, 1)
    p = Pipeline(gpu_ctx, w.config(), w.grid(1), 1, b.n_hits, 500_000, 500_000, 100_000)
    trk, off, _ = p.seed(b)
    lt0, lt1 = trk[off[0]:off[1]], trk[off[1]:off[2]]
    bt = TrackletCollection.from_host(gpu_ctx, lt0)
    ft = TrackletCollection.from_host(gpu_ctx, lt1)
    TripletConnectivity(gpu_ctx).run(bt, ft, tight_packing=True)
    gpu_ctx.synchronize()
    want = oracle.connectivity(lt0, np.zeros(len(lt0), np.uint32), lt1,
                               np.zeros(len(lt1), np.uint32), tight_packing=True)
    got = ft.get_connectivity()
    assert np.array_equal(got, want)
    assert (got > 0).sum() > 0.5 * len(lt1)  # most (2,3,4) seeds continue a (1,2,3) seed
