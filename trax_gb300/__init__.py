"""trax-gb300: GB300-native triplet seeding (grid build -> pairs -> predict -> filter).

The compute path is libtrax_gb300.so (hand-written sm_103a CUDA behind the
C-ABI in include/trax.h).  This package is its host-side binding and the
reference-shaped operator classes; there is no CPU fallback.
"""
from ._abi import (TraxConfig, TraxGridCfg, TraxLayerTriplet, make_config)  # noqa: F401
from .runtime import Context, TraxError, load_library, LIB_PATH, EXPORTED_SYMBOLS  # noqa: F401
from .ops import (EventSupplement, LayerSupplement, HitCollection, Grid, Pairing,  # noqa: F401
                  TrackletCollection, GridBuilder, PairGeneratorBeamspot, PairGeneratorSector,
                  TripletThetaPhiPredictor, TripletThetaPhiFilter, TripletConnectivity,
                  Pipeline, build_triplets,
                  supplements)
from . import gen  # noqa: F401
