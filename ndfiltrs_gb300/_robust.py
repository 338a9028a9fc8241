"""Local percentiles (``percentile_filter`` / ``nanpercentile_filter``).

Same signatures and semantics as the reference's percentile API
(python/ndfiltrs/_robust.py:31-176 of ysBach/ndfiltrs v0.2.0): linear
interpolation at rank ``(n - 1) * q / 100`` of the retained samples, computed
in float64 and cast once. Selection of the two ranks runs on the GPU. The
other robust statistics of the reference (MAD, sigma clipping, mode,
biweight) are outside this library's scope.
"""

from __future__ import annotations

import math
import numbers

import numpy as np
from numpy.typing import ArrayLike

from . import _core
from ._api import BoundaryMode, FloatArray
from ._validation import check_flag, validate


def _finite_real(value: object, name: str) -> float:
    if isinstance(value, (bool, np.bool_)) or not isinstance(value, numbers.Real):
        raise TypeError(f"{name} must be a non-boolean real number")
    number = float(value)
    if not math.isfinite(number):
        raise ValueError(f"{name} must be finite")
    return number


def _percentile(value: object) -> float:
    q = _finite_real(value, "percentile")
    if not 0 <= q <= 100:
        raise ValueError("percentile must lie between 0 and 100")
    return q


def _call(args, q: float, omit_nan: bool, ignore_inf: bool, min_count: int) -> FloatArray:
    return _core.robust_filter(
        args.array,
        args.size,
        args.footprint,
        args.origin,
        args.mode,
        args.cval,
        kind="percentile",
        parameter=q,
        omit_nan=omit_nan,
        ignore_inf=ignore_inf,
        min_count=min_count,
        sigma_lower=3.0,
        sigma_upper=3.0,
        maxiters=5,
        center="median",
        spread="std",
    )


def percentile_filter(
    array: ArrayLike,
    percentile: float,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """Linearly interpolated percentile of each window; NaNs propagate."""
    q = _percentile(percentile)
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _call(args, q, False, False, 1)


def nanpercentile_filter(
    array: ArrayLike,
    percentile: float,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """Percentile of the retained samples; windows below ``min_count`` give
    canonical NaN."""
    q = _percentile(percentile)
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _call(args, q, True, bool(ignore_inf), args.min_count)
