"""GB300-native (sm_103a) Tb.Th / Tb.Sp hot path of bone-morphometry.

The exact squared EDT and the distance-ridge + sphere-fill local thickness of
the reference (src/edt.rs, src/local_thickness.rs), their Tb.Th / Tb.Sp
statistics (src/metrics.rs) and the batched / served forms, computed by
hand-written CUDA kernels behind the C ABI of include/bm.h.
"""

from ._lib import BoneMorphometryError, Context, default_context, library_path, load
from .api import (BinaryVolume, DistributionStats, FeatureMode, Phase, ThicknessMetrics, analyze_thickness,
                  euclidean_distance_transform_squared, local_thickness, nonzero_stats, volume_metrics)

__all__ = [
    "BinaryVolume", "BoneMorphometryError", "Context", "DistributionStats", "FeatureMode", "Phase",
    "ThicknessMetrics", "analyze_thickness", "default_context", "euclidean_distance_transform_squared",
    "library_path", "load", "local_thickness", "nonzero_stats", "volume_metrics",
]
