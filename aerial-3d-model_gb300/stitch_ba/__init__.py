"""GB300-native GPS-aided bundle adjustment: the drop-in for stitch-core's
``recon::ba::bundle_adjust`` (crates/stitch-core/src/recon/ba.rs:198)."""
from .problem import BaStats, Intrinsics, Obs, Problem  # noqa: F401
from .ba import (Context, Options, PairMatches, SolveInfo, SparseSummary,  # noqa: F401
                 Tracks, bundle_adjust, bundle_adjust_batch, pair_fits, ransac_fundamental,
                 sparse_summary, triangulate)
from .native import BaError  # noqa: F401
