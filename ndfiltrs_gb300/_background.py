"""Mesh (grid) background and RMS estimation (``mesh_background``).

Same signature, defaults, validation and result as the reference's
``python/ndfiltrs/_background.py`` (ysBach/ndfiltrs v0.2.0): the per-mesh
statistics and the full-resolution maps run on the GPU (``mesh.cu``); fill and
median filter of the small mesh grid run on the host. Statistics are float64;
maps are cast once to the input dtype.
"""

from __future__ import annotations

from collections.abc import Sequence
from typing import NamedTuple

import numpy as np
from numpy.typing import ArrayLike, NDArray

from . import _core
from ._robust import _finite_real, _pearson
from ._validation import as_index, check_array

FloatArray = NDArray[np.float32] | NDArray[np.float64]


class MeshBackground(NamedTuple):
    """Result of `mesh_background`: full-resolution maps, the float64 mesh
    grids after fill and median filter, validity (before fill), per-mesh
    finite and retained counts, and the medians of the two grids."""

    background: FloatArray
    rms: FloatArray
    mesh_background: NDArray[np.float64]
    mesh_rms: NDArray[np.float64]
    mesh_valid: NDArray[np.bool_]
    mesh_finite_count: NDArray[np.int64]
    mesh_retained_count: NDArray[np.int64]
    global_background: float
    global_rms: float


def _sizes(value: object, ndim: int, name: str, *, odd: bool) -> tuple[int, ...]:
    """A positive integer broadcast to every axis, or one entry per axis."""
    message = f"{name} must be an integer or a sequence of integers"
    if isinstance(value, np.ndarray) and value.ndim == 1:
        value = value.tolist()
    if isinstance(value, Sequence) and not isinstance(value, (str, bytes)):
        sizes = tuple(as_index(entry, message) for entry in value)
        if len(sizes) != ndim:
            raise ValueError(f"{name} must have one entry per array dimension")
    else:
        sizes = (as_index(value, message),) * ndim
    if any(size <= 0 for size in sizes):
        raise ValueError(f"{name} entries must be positive")
    if odd and any(size % 2 == 0 for size in sizes):
        raise ValueError(f"{name} entries must be odd")
    return sizes


def _choice(value: object, name: str, options: tuple[str, ...]) -> str:
    if not isinstance(value, str) or value not in options:
        raise ValueError(f"{name} must be one of {options}")
    return value


def mesh_background(
    data: ArrayLike,
    box_size: int | Sequence[int],
    *,
    mask: ArrayLike | None = None,
    filter_size: int | Sequence[int] = 3,
    estimator: str = "sextractor",
    sigma: float = 3.0,
    sigma_lower: float | None = None,
    sigma_upper: float | None = None,
    maxiters: int | None = 10,
    center: str = "median",
    spread: str = "std",
    statistic: str = "mode",
    mode_estimator: str = "sex",
    pearson: float | None = None,
    rms: str = "std",
    min_valid_fraction: float = 0.5,
    valid_count: str = "finite",
    valid_base: str = "mesh",
    fill: str = "nearest",
    idw_neighbors: int = 10,
    idw_power: float = 1.0,
    filter_edge: str = "shrink",
    filter_threshold: float | None = None,
    threshold_kind: str = "deviation",
    interpolation: str = "spline",
) -> MeshBackground:
    """Estimate smooth background and RMS maps from a grid of meshes.

    Each mesh (``box_size``, partial at the far edges) gets a robust
    background and RMS from its finite, unmasked samples ('sextractor': the
    SExtractor sequence on exact samples; 'sigma_clip': one iterative clip and
    its statistic). Meshes failing ``min_valid_fraction`` are filled from valid
    meshes ('nearest' or 'idw'), the grid is median filtered
    (``filter_size``, 'shrink' or 'truncate' edges, optional threshold), and a
    natural cubic spline ('spline') or the SExtractor-compatible form
    ('sextractor', 2-D) maps it to full resolution. Defaults follow
    SExtractor.
    """
    value = check_array(data)
    ndim = value.ndim
    boxes = _sizes(box_size, ndim, "box_size", odd=False)
    filters = _sizes(filter_size, ndim, "filter_size", odd=True)
    if mask is not None:
        if np.ma.isMaskedArray(mask):
            raise TypeError("mask must not be a masked array")
        flags = np.asarray(mask)
        if flags.dtype.kind not in "biuf":
            raise TypeError("mask must have a boolean or real numeric dtype")
        if flags.shape != value.shape:
            raise ValueError("mask must have the same shape as data")
        mask = np.ascontiguousarray(flags != 0)
    estimator = _choice(estimator, "estimator", ("sextractor", "sigma_clip"))
    lower = _finite_real(sigma if sigma_lower is None else sigma_lower, "sigma_lower")
    upper = _finite_real(sigma if sigma_upper is None else sigma_upper, "sigma_upper")
    if maxiters is not None:
        maxiters = as_index(maxiters, "maxiters must be an integer or None")
        if maxiters < 0:
            raise ValueError("maxiters must be nonnegative")
    mode_estimator = _choice(mode_estimator, "mode_estimator", ("sex", "mmm", "iraf"))
    # The SExtractor estimator always uses the 'sex' rule.
    factor = _pearson("sex" if estimator == "sextractor" else mode_estimator, pearson)
    neighbors = as_index(idw_neighbors, "idw_neighbors must be an integer")
    threshold = None if filter_threshold is None else _finite_real(filter_threshold, "filter_threshold")
    value = np.require(value, dtype=value.dtype, requirements=("C", "A"))
    outputs = _core.mesh_background(
        value,
        mask,
        boxes,
        filters,
        estimator,
        lower,
        upper,
        maxiters,
        _choice(center, "center", ("median", "mean")),
        _choice(spread, "spread", ("std", "mad")),
        _choice(statistic, "statistic", ("mode", "mean", "median")),
        mode_estimator,
        factor,
        _choice(rms, "rms", ("std", "mad")),
        _finite_real(min_valid_fraction, "min_valid_fraction"),
        _choice(valid_count, "valid_count", ("finite", "retained")),
        _choice(valid_base, "valid_base", ("mesh", "box")),
        _choice(fill, "fill", ("nearest", "idw")),
        neighbors,
        _finite_real(idw_power, "idw_power"),
        _choice(filter_edge, "filter_edge", ("shrink", "truncate")),
        threshold,
        _choice(threshold_kind, "threshold_kind", ("deviation", "above")),
        _choice(interpolation, "interpolation", ("spline", "sextractor")),
    )
    return MeshBackground(*outputs)
