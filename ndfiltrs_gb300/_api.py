"""Public window-filter API of ndfiltrs_gb300.

Signatures, defaults and semantics match the reference's public functions
(python/ndfiltrs/_api.py:86-1028 of ysBach/ndfiltrs v0.2.0), so code written
against ``ndfiltrs`` runs unchanged. Every function validates its arguments
and calls ``_core.window_filter``, which runs on the GPU.

``method`` keeps the reference's meaning as an exact-algorithm choice whose
results are identical across methods. On the GPU, "direct" and "sortnet"
both run per-thread register selection (a sorting network over the halo
tile), and "histogram" runs the sliding rank-histogram kernel for
rectangular 1-D/2-D windows; windows too wide for a register network use the
histogram kernel (rectangular) or a radix select (footprints).

``mean_filter`` / ``nanmean_filter(method="boxcar")`` run the exact rolling
mean (kind "mean_rolling"): the window's finite samples summed exactly and the
mean rounded once. ``method="separable"`` (the reference's separable
float64 mean) is outside this path and raises NotImplementedError.
"""

from __future__ import annotations

from typing import Literal

import numpy as np
from numpy.typing import ArrayLike, NDArray

from . import _core
from ._validation import Arguments, as_index, check_flag, check_method, validate

BoundaryMode = Literal["reflect", "constant", "nearest", "mirror", "wrap"]
FloatArray = NDArray[np.float32] | NDArray[np.float64]


def _run(kind: str, args: Arguments, *, ignore_inf: bool | None = None, parameter: int = 0) -> FloatArray:
    """One native reduction; ``ignore_inf=None`` selects the propagate policy."""
    return _core.window_filter(
        args.array,
        kind,
        args.size,
        args.footprint,
        args.origin,
        args.mode,
        args.cval,
        ignore_inf is not None,
        bool(ignore_inf),
        args.min_count,
        parameter,
    )


def _median_kind(method: object, args: Arguments) -> str:
    check_method(method, ("direct", "sortnet", "histogram"))
    if method == "histogram" and args.footprint is not None:
        raise ValueError("method='histogram' requires size, not footprint")
    return {"direct": "median", "sortnet": "median_network", "histogram": "median_histogram"}[
        str(method)
    ]


def _mean_kind(method: object, args: Arguments) -> str:
    check_method(method, ("direct", "separable", "boxcar"))
    if method == "boxcar" and args.footprint is not None:
        raise ValueError("method='boxcar' requires size, not footprint")
    if method == "separable":
        raise NotImplementedError(
            "mean method 'separable' is outside this library's scope; use 'direct' or 'boxcar'"
        )
    return "mean_rolling" if method == "boxcar" else "mean"


def median_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    method: Literal["direct", "sortnet", "histogram"] = "direct",
) -> FloatArray:
    """N-dimensional median filter; NaNs propagate, infinities take part.

    An even window count gives the float64 midpoint of the two middle values
    (cast once to the dtype), unlike SciPy which returns the upper one.
    """
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _run(_median_kind(method, args), args)


def nanmedian_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
    method: Literal["direct", "sortnet", "histogram"] = "direct",
) -> FloatArray:
    """Median filter that omits NaNs (and infinities with ``ignore_inf``).

    Windows with fewer than ``min_count`` retained samples give canonical NaN.
    """
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _run(_median_kind(method, args), args, ignore_inf=bool(ignore_inf))


def mean_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    method: Literal["direct", "separable", "boxcar"] = "direct",
) -> FloatArray:
    """Arithmetic mean of each window; NaNs propagate locally."""
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _run(_mean_kind(method, args), args)


def nanmean_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
    method: Literal["direct", "separable", "boxcar"] = "direct",
) -> FloatArray:
    """Mean of each window omitting NaNs (and infinities with ``ignore_inf``)."""
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _run(_mean_kind(method, args), args, ignore_inf=bool(ignore_inf))


def min_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """Minimum in IEEE total order (-0.0 before +0.0); NaNs propagate."""
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _run("min", args)


def max_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
) -> FloatArray:
    """Maximum in IEEE total order; NaNs propagate."""
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    return _run("max", args)


def nanmin_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """Minimum of the retained samples of each window."""
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _run("min", args, ignore_inf=bool(ignore_inf))


def nanmax_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """Maximum of the retained samples of each window."""
    check_flag(ignore_inf, "ignore_inf")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count)
    return _run("max", args, ignore_inf=bool(ignore_inf))


def var_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ddof: int = 0,
) -> FloatArray:
    """Window variance with ``ddof`` delta degrees of freedom."""
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1, ddof=ddof)
    return _run("var", args, parameter=args.ddof)


def std_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ddof: int = 0,
) -> FloatArray:
    """Window standard deviation with ``ddof`` delta degrees of freedom."""
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1, ddof=ddof)
    return _run("std", args, parameter=args.ddof)


def nanvar_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ddof: int = 0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """Variance of the retained samples of each window."""
    check_flag(ignore_inf, "ignore_inf")
    args = validate(
        array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count, ddof=ddof
    )
    return _run("var", args, ignore_inf=bool(ignore_inf), parameter=args.ddof)


def nanstd_filter(
    array: ArrayLike,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    ddof: int = 0,
    ignore_inf: bool = False,
    min_count: int = 1,
) -> FloatArray:
    """Standard deviation of the retained samples of each window."""
    check_flag(ignore_inf, "ignore_inf")
    args = validate(
        array, size, mode, cval, footprint=footprint, origin=origin, min_count=min_count, ddof=ddof
    )
    return _run("std", args, ignore_inf=bool(ignore_inf), parameter=args.ddof)


def rank_filter(
    array: ArrayLike,
    rank: int,
    size: int | tuple[int, ...] | None = None,
    *,
    footprint: ArrayLike | None = None,
    origin: int | tuple[int, ...] = 0,
    mode: BoundaryMode | tuple[BoundaryMode, ...] = "reflect",
    cval: float = 0.0,
    method: Literal["direct", "histogram"] = "direct",
) -> FloatArray:
    """Value of zero-based ``rank`` in each sorted window (negative counts
    from the maximum); NaNs propagate."""
    position = as_index(rank, "rank must be an integer, not a boolean")
    args = validate(array, size, mode, cval, footprint=footprint, origin=origin, min_count=1)
    if not -args.count <= position < args.count:
        raise ValueError("rank must satisfy -n <= rank < n for n window elements")
    check_method(method, ("direct", "histogram"))
    if method == "histogram" and args.footprint is not None:
        raise ValueError("method='histogram' requires size, not footprint")
    return _run(
        "rank_histogram" if method == "histogram" else "rank",
        args,
        parameter=position % args.count,
    )


def get_num_threads() -> int:
    """Return the number of threads in the library's host-side pool.

    As with the reference's global Rayon pool, ``RAYON_NUM_THREADS`` (set
    before the first call of the process) fixes it; the default is the
    hardware thread count capped at 16. Device work always spans every SM.
    """
    return _core.get_num_threads()
