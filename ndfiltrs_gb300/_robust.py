"""Local percentiles, median absolute deviations, sigma-clipped statistics,
modes and biweight estimates.

Same signatures and semantics as the reference's robust API
(python/ndfiltrs/_robust.py of ysBach/ndfiltrs v0.2.0). Percentiles select
their two ranks on the GPU and interpolate in float64; the MAD, clipping,
mode and biweight filters run the reference's float64 estimators per window
on the GPU (``robust.cu``). Every result is cast once to the input dtype.
"""

from __future__ import annotations

import math
import numbers

import numpy as np
from numpy.typing import ArrayLike

from . import _core
from ._api import BoundaryMode, FloatArray
from ._validation import as_index, check_flag, validate

_MODE_ESTIMATORS = ("sex", "mmm", "iraf")


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


def _robust(args, kind: str, *, omit_nan: bool, ignore_inf: bool = False, parameter: float = 0.0,
            sigma_lower: float = 3.0, sigma_upper: float = 3.0, maxiters: int | None = 5,
            center: str = "median", spread: str = "std", estimator: str = "sex",
            modify_sample_size: bool = False, pearson: float = 2.5) -> FloatArray:
    return _core.robust_filter(
        args.array,
        args.size,
        args.footprint,
        args.origin,
        args.mode,
        args.cval,
        kind=kind,
        parameter=parameter,
        omit_nan=omit_nan,
        ignore_inf=ignore_inf,
        min_count=args.min_count,
        sigma_lower=sigma_lower,
        sigma_upper=sigma_upper,
        maxiters=maxiters,
        center=center,
        spread=spread,
        estimator=estimator,
        modify_sample_size=modify_sample_size,
        pearson=pearson,
    )


def _scale(value: object) -> float:
    multiplier = _finite_real(value, "scale")
    if multiplier < 0:
        raise ValueError("scale must be nonnegative")
    return multiplier


def _positive_finite(value: object, name: str) -> float:
    number = _finite_real(value, name)
    if number <= 0:
        raise ValueError(f"{name} must be positive")
    return number


def _pearson(estimator: object, pearson: object) -> float:
    """The mode rule's Pearson factor (2.5 for 'sex', 3 otherwise)."""
    if not isinstance(estimator, str) or estimator not in _MODE_ESTIMATORS:
        raise ValueError(f"mode_estimator must be one of {_MODE_ESTIMATORS}")
    if pearson is None:
        return 2.5 if estimator == "sex" else 3.0
    factor = _finite_real(pearson, "pearson")
    if factor < 1:
        raise ValueError("pearson must be at least 1")
    return factor


def mad_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    scale: float = 1.0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """``scale * median(|x - median(x)|)`` of each window; NaNs propagate,
    infinities participate (an undefined deviation gives NaN)."""
    multiplier = _scale(scale)
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _robust(args, "mad", omit_nan=False, parameter=multiplier)


def nanmad_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    scale: float = 1.0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """The MAD of the retained samples (NaNs omitted, infinities too with
    ``ignore_inf``); windows below ``min_count`` give canonical NaN."""
    multiplier = _scale(scale)
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _robust(args, "mad", omit_nan=True, ignore_inf=bool(ignore_inf), parameter=multiplier)


def sigma_clipped_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    sigma: float = 3.0,
    sigma_lower: float | None = None,
    sigma_upper: float | None = None,
    maxiters: int | None = 5,
    center: str = "median",
    spread: str = "std",
    statistic: str = "mean",
    mode_estimator: str = "sex",
    pearson: float | None = None,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    min_count: int = 1,
) -> FloatArray:
    """Iterative clipping of each window's finite samples to
    ``[center - sigma_lower * spread, center + sigma_upper * spread]``, then
    the mean, median or mode of what remains (``min_count`` checked after
    clipping)."""
    threshold = _finite_real(sigma, "sigma")
    lower = threshold if sigma_lower is None else _finite_real(sigma_lower, "sigma_lower")
    upper = threshold if sigma_upper is None else _finite_real(sigma_upper, "sigma_upper")
    if threshold < 0 or lower < 0 or upper < 0:
        raise ValueError("sigma and its lower and upper overrides must be nonnegative")
    iterations = None
    if maxiters is not None:
        iterations = as_index(maxiters, "maxiters must be an integer, not a boolean")
        if iterations < 0:
            raise ValueError("maxiters must be nonnegative")
        if iterations > np.iinfo(np.int64).max:
            raise OverflowError("maxiters exceeds the native index range")
    for name, value, choices in (
        ("center", center, ("mean", "median")),
        ("spread", spread, ("std", "mad")),
        ("statistic", statistic, ("mean", "median", "mode")),
    ):
        if not isinstance(value, str) or value not in choices:
            raise ValueError(f"{name} must be one of {choices}")
    factor = _pearson(mode_estimator, pearson)
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _robust(args, f"sigma_{statistic}", omit_nan=True, ignore_inf=True, sigma_lower=lower,
                   sigma_upper=upper, maxiters=iterations, center=center, spread=spread,
                   estimator=mode_estimator, pearson=factor)


def mode_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode_estimator: str = "sex",
    pearson: float | None = None,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """Mode estimate from each window's mean, median and population std
    ('sex', 'mmm' or 'iraf' rule); windows holding NaN or infinity give NaN."""
    factor = _pearson(mode_estimator, pearson)
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _robust(args, "mode", omit_nan=False, estimator=mode_estimator, pearson=factor,
                   maxiters=None)


def nanmode_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode_estimator: str = "sex",
    pearson: float | None = None,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """The mode estimate of the retained samples (NaNs omitted)."""
    factor = _pearson(mode_estimator, pearson)
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _robust(args, "mode", omit_nan=True, ignore_inf=bool(ignore_inf), estimator=mode_estimator,
                   pearson=factor, maxiters=None)


def biweight_location_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    c: float = 6.0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """Tukey's biweight location about each window's median."""
    tuning = _positive_finite(c, "c")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _robust(args, "biweight_location", omit_nan=False, parameter=tuning, maxiters=None)


def nanbiweight_location_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    c: float = 6.0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """The biweight location of the retained samples (NaNs omitted)."""
    tuning = _positive_finite(c, "c")
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _robust(args, "biweight_location", omit_nan=True, ignore_inf=bool(ignore_inf),
                   parameter=tuning, maxiters=None)


def biweight_scale_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    c: float = 9.0,
    modify_sample_size: bool = False,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """The biweight scale (square root of the biweight midvariance)."""
    check_flag(modify_sample_size, "modify_sample_size")
    tuning = _positive_finite(c, "c")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _robust(args, "biweight_scale", omit_nan=False, parameter=tuning,
                   modify_sample_size=bool(modify_sample_size), maxiters=None)


def nanbiweight_scale_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    c: float = 9.0,
    modify_sample_size: bool = False,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """The biweight scale of the retained samples (NaNs omitted)."""
    check_flag(modify_sample_size, "modify_sample_size")
    tuning = _positive_finite(c, "c")
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _robust(args, "biweight_scale", omit_nan=True, ignore_inf=bool(ignore_inf),
                   parameter=tuning, modify_sample_size=bool(modify_sample_size), maxiters=None)
