"""Footprint generators for window filters: ``box``, ``tophat`` and ``ring``.

Same definitions as the reference's kernel constructors
(python/ndfiltrs/kernels.py:309-395 of ysBach/ndfiltrs v0.2.0): the weight
of a pixel is the fraction of its ``oversample**ndim`` subpixel centers that
fall inside the region (a ball of ``radius`` for ``tophat``; the inclusive
shell ``radius_in <= r <= radius_out`` for ``ring``), the array is cropped to
the smallest support that keeps every nonzero weight, and ``normalize``
divides by the sum. Use ``kernel != 0`` as a footprint.
"""

from __future__ import annotations

import itertools
import math
import numbers
from collections.abc import Sequence

import numpy as np
from numpy.typing import NDArray


def _positive_int(value: object, name: str) -> int:
    if isinstance(value, (bool, np.bool_)) or not isinstance(value, numbers.Integral):
        raise TypeError(f"{name} must be an integer")
    value = int(value)
    if value < 1:
        raise ValueError(f"{name} must be positive")
    return value


def _radius(value: object, name: str) -> float:
    if isinstance(value, (bool, np.bool_)) or not isinstance(value, numbers.Real):
        raise TypeError(f"{name} must be a real number")
    value = float(value)
    if not math.isfinite(value) or value < 0:
        raise ValueError(f"{name} must be finite and nonnegative")
    return value


def _finish(weights: NDArray[np.float64], normalize: bool) -> NDArray[np.float64]:
    if normalize:
        total = weights.sum()
        if total == 0:
            raise ValueError("kernel weights sum to zero")
        weights = weights / total
    return np.ascontiguousarray(weights, dtype=np.float64)


def _shell_fraction(extent: int, ndim: int, oversample: int, inner: float, outer: float) -> NDArray[np.float64]:
    side = 2 * extent + 1
    grid = np.arange(-extent, extent + 1, dtype=np.float64)
    # Subpixel centers at (k + 1/2) / f - 1/2 inside each pixel.
    shifts = (np.arange(oversample, dtype=np.float64) + 0.5) / oversample - 0.5
    total = np.zeros((side,) * ndim, dtype=np.float64)
    for offset in itertools.product(shifts, repeat=ndim):
        distance2 = np.zeros((side,) * ndim, dtype=np.float64)
        for axis in range(ndim):
            coordinate = grid + offset[axis]
            shape = [1] * ndim
            shape[axis] = side
            distance2 = distance2 + (coordinate * coordinate).reshape(shape)
        total += (distance2 >= inner * inner) & (distance2 <= outer * outer)
    return total / oversample**ndim


def _crop(weights: NDArray[np.float64], extent: int) -> NDArray[np.float64]:
    nonzero = np.argwhere(weights != 0)
    if nonzero.size == 0:
        raise ValueError("no subpixel sample lies inside the region; widen it or increase oversample")
    keep = [int(np.max(np.abs(nonzero[:, axis] - extent))) for axis in range(weights.ndim)]
    return weights[tuple(slice(extent - k, extent + k + 1) for k in keep)]


def box(size: int | Sequence[int], ndim: int | None = None, *, normalize: bool = True) -> NDArray[np.float64]:
    """Uniform box of ``size`` pixels per axis (a scalar size needs ``ndim``)."""
    if isinstance(size, numbers.Integral) and not isinstance(size, (bool, np.bool_)):
        if ndim is None:
            raise TypeError("ndim is required when size is scalar")
        sizes = (_positive_int(size, "size"),) * _positive_int(ndim, "ndim")
    else:
        if isinstance(size, (str, bytes, bool, np.bool_)):
            raise TypeError("size must be an integer or a sequence of integers")
        sizes = tuple(_positive_int(v, "size entries") for v in size)
        if not sizes:
            raise ValueError("size must contain at least one value")
        if ndim is not None and _positive_int(ndim, "ndim") != len(sizes):
            raise ValueError("ndim must match the length of size")
    return _finish(np.ones(sizes, dtype=np.float64), bool(normalize))


def tophat(radius: float, ndim: int, *, oversample: int = 1, normalize: bool = True) -> NDArray[np.float64]:
    """Pixel fractions inside an ``ndim``-ball of ``radius`` (boundary included)."""
    outer = _radius(radius, "radius")
    ndim = _positive_int(ndim, "ndim")
    factor = _positive_int(oversample, "oversample")
    extent = max(0, math.floor(outer + 0.5 - 0.5 / factor))
    weights = _shell_fraction(extent, ndim, factor, 0.0, outer)
    return _finish(_crop(weights, extent), bool(normalize))


def ring(
    radius_in: float,
    radius_out: float,
    ndim: int,
    *,
    oversample: int = 1,
    normalize: bool = True,
) -> NDArray[np.float64]:
    """Pixel fractions in the inclusive shell ``radius_in <= r <= radius_out``."""
    inner = _radius(radius_in, "radius_in")
    outer = _radius(radius_out, "radius_out")
    if outer < inner:
        raise ValueError("radius_out must be greater than or equal to radius_in")
    ndim = _positive_int(ndim, "ndim")
    factor = _positive_int(oversample, "oversample")
    extent = max(0, math.floor(outer + 0.5 - 0.5 / factor))
    weights = _shell_fraction(extent, ndim, factor, inner, outer)
    return _finish(_crop(weights, extent), bool(normalize))
