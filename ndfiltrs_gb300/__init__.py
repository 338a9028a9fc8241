"""ndfiltrs_gb300 — GB300-native (CUDA sm_103a) windowed statistics.

A drop-in for the windowed-statistics path of ndfiltrs (ysBach/ndfiltrs
v0.2.0): NaN-aware median, rank and percentile filters (direct, sortnet and
histogram methods), the mean/var/std footprint reductions, exact rolling
means, separable min/max and the robust family (MAD, sigma clipping, mode,
biweight), for every footprint, origin and boundary mode, and the mesh
background built on them. The public functions keep the reference's
signatures and NaN/inf/min_count semantics; all computation runs on the GPU
through the C-ABI library ``libndfiltrs_gb300.so``.
"""

from . import kernels
from ._api import (
    get_num_threads,
    max_filter,
    mean_filter,
    median_filter,
    min_filter,
    nanmax_filter,
    nanmean_filter,
    nanmedian_filter,
    nanmin_filter,
    nanstd_filter,
    nanvar_filter,
    rank_filter,
    std_filter,
    var_filter,
)
from ._background import MeshBackground, mesh_background
from ._core import Batch, Plan, autotune_entries, device_info, set_autotune
from ._robust import (
    biweight_location_filter,
    biweight_scale_filter,
    mad_filter,
    mode_filter,
    nanbiweight_location_filter,
    nanbiweight_scale_filter,
    nanmad_filter,
    nanmode_filter,
    nanpercentile_filter,
    percentile_filter,
    sigma_clipped_filter,
)

__all__ = [
    "Batch",
    "Plan",
    "autotune_entries",
    "biweight_location_filter",
    "biweight_scale_filter",
    "device_info",
    "get_num_threads",
    "kernels",
    "mad_filter",
    "mesh_background",
    "MeshBackground",
    "max_filter",
    "mean_filter",
    "median_filter",
    "min_filter",
    "mode_filter",
    "nanbiweight_location_filter",
    "nanbiweight_scale_filter",
    "nanmad_filter",
    "nanmax_filter",
    "nanmean_filter",
    "nanmedian_filter",
    "nanmin_filter",
    "nanmode_filter",
    "nanpercentile_filter",
    "nanstd_filter",
    "nanvar_filter",
    "percentile_filter",
    "rank_filter",
    "set_autotune",
    "sigma_clipped_filter",
    "std_filter",
    "var_filter",
]
__version__ = "0.1.0"
