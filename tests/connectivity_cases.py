"""The reference's TripletConnectivity known-answer tables
(src/algorithms/test/TripletConnectivityTest.h:22-108) and expected results
(:147-259).  Rows are (hit1, hit2, hit3); connectivity starts at 0."""

SIMPLE_FORWARD = {  # addSimpleForward, test_run
    "base": [(1, 2, 3), (1, 2, 4)],
    "following": [(3, 5, 6), (9, 4, 8)],
    "expect_following": [1, 0],
}

SIMPLE_BACKWARD = {  # addSimpleBackward, test_run_backward
    "base": [(3, 2, 23), (5, 2, 1)],
    "following": [(12, 8, 3), (15, 11, 8)],
    "expect_following": [1, 0],
}

FOUR_LAYER = [  # addFourLayerForward, test_run_multilayer (expects layer 4)
    [(1, 3, 8), (1, 3, 5), (2, 4, 6), (2, 4, 7)],
    [(6, 11, 16), (9, 12, 17), (9, 13, 18), (9, 14, 19)],
    [(16, 21, 30), (15, 22, 29), (15, 24, 29), (15, 25, 27)],
    [(30, 31, 36), (28, 32, 37), (26, 33, 38), (27, 34, 39)],
]
FOUR_LAYER_EXPECT = [3, 0, 0, 1]

FOUR_LAYER_TIGHT = [  # addFourLayerForwardTight, test_run_tight_multilayer
    [(1, 4, 6), (1, 3, 5), (2, 3, 8), (2, 4, 7)],
    [(4, 6, 16), (9, 12, 17), (9, 13, 18), (9, 14, 19)],
    [(6, 16, 30), (15, 22, 29), (15, 24, 29), (15, 25, 27)],
    [(16, 30, 36), (28, 32, 37), (26, 33, 38), (27, 34, 39)],
]
FOUR_LAYER_TIGHT_EXPECT = [3, 0, 0, 0]
