"""TripletConnectivity oracle against the reference's own known answers."""
import numpy as np

import oracle
from connectivity_cases import (FOUR_LAYER, FOUR_LAYER_EXPECT, FOUR_LAYER_TIGHT,
                                FOUR_LAYER_TIGHT_EXPECT, SIMPLE_BACKWARD, SIMPLE_FORWARD)


def _chain(layers, tight):
    con = np.zeros(len(layers[0]), np.uint32)
    for base, follow in zip(layers[:-1], layers[1:]):
        con = oracle.connectivity(base, con, follow, np.zeros(len(follow), np.uint32),
                                  tight_packing=tight)
    return con.tolist()


def test_simple_forward_and_backward():
    c = SIMPLE_FORWARD
    assert oracle.connectivity(c["base"], [0, 0], c["following"], [0, 0]).tolist() == \
        c["expect_following"]
    c = SIMPLE_BACKWARD
    assert oracle.connectivity(c["base"], [0, 0], c["following"], [0, 0],
                               iterate_backwards=True).tolist() == c["expect_following"]


def test_four_layer_chains():
    assert _chain(FOUR_LAYER, tight=False) == FOUR_LAYER_EXPECT
    assert _chain(FOUR_LAYER_TIGHT, tight=True) == FOUR_LAYER_TIGHT_EXPECT


def test_literal_wide_kernel_disagrees_with_reference_test():
    """The wide kernel as written (base indexed by the following id) passes
    the two-tracklet tests but gives 2, not the tested 3, for the track."""
    c = SIMPLE_FORWARD
    lit = oracle.connectivity_literal_wide([r[2] for r in c["base"]], [0, 0],
                                           [r[0] for r in c["following"]], [0, 0])
    assert lit.tolist() == c["expect_following"]
    con = np.zeros(4, np.uint32)
    for base, follow in zip(FOUR_LAYER[:-1], FOUR_LAYER[1:]):
        con = oracle.connectivity_literal_wide([r[2] for r in base], con,
                                               [r[0] for r in follow], np.zeros(4, np.uint32))
    assert con.tolist() == [2, 0, 0, 1] != FOUR_LAYER_EXPECT
