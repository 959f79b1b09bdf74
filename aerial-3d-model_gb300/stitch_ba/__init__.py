"""GB300-native GPS-aided bundle adjustment: the drop-in for stitch-core's
``recon::ba::bundle_adjust`` (crates/stitch-core/src/recon/ba.rs:198)."""
from .problem import BaStats, Intrinsics, Obs, Problem  # noqa: F401
from .ba import (Context, Options, SolveInfo, SparseSummary, Tracks,  # noqa: F401
                 bundle_adjust, bundle_adjust_batch, sparse_summary, triangulate)
from .native import BaError  # noqa: F401
