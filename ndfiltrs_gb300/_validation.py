"""Argument validation of the public API.

The rules and messages match the reference's public contract
(python/ndfiltrs/_validation.py:16-211 and docs/semantics.md of
ysBach/ndfiltrs v0.2.0) so that callers see the same exceptions:

* the array: no masked arrays, rank >= 1, native-endian float32/float64,
  aligned; normalized to an owned C-contiguous array when needed;
* ``size`` (integer-index protocol, booleans rejected) or ``footprint``
  (nonzero entries selected), mutually exclusive, default 3 per axis;
* ``origin`` per axis within ``-(n // 2) <= origin <= (n - 1) // 2``;
* ``mode`` names per axis; ``cval`` a non-boolean real cast to the dtype;
* ``min_count`` between 1 and the selected element count; ``ddof >= 0``.
"""

from __future__ import annotations

import numbers
import operator
from collections.abc import Sequence
from dataclasses import dataclass

import numpy as np

MODES = ("reflect", "constant", "nearest", "mirror", "wrap")
_INDEX_MAX = int(np.iinfo(np.uintp).max)


@dataclass(frozen=True)
class Arguments:
    """Normalized inputs of one native call."""

    array: np.ndarray
    size: tuple[int, ...]
    footprint: list[bool] | None
    origin: tuple[int, ...]
    mode: tuple[str, ...]
    cval: float
    min_count: int
    ddof: int
    count: int


def as_index(value: object, message: str) -> int:
    """Integer-index protocol without booleans."""
    if isinstance(value, (bool, np.bool_)):
        raise TypeError(message)
    try:
        return operator.index(value)
    except TypeError:
        raise TypeError(message) from None


def check_array(array: object) -> np.ndarray:
    if np.ma.isMaskedArray(array):
        raise TypeError("masked arrays are not supported")
    value = np.asarray(array)
    if value.ndim == 0:
        raise ValueError("array must have at least one dimension")
    if value.dtype.kind != "f" or value.dtype.itemsize not in (4, 8):
        raise TypeError("array dtype must be float32 or float64")
    if not value.dtype.isnative:
        raise TypeError("array dtype must be native-endian")
    if not value.flags.aligned:
        raise ValueError("array must be aligned")
    return value


def _sizes(size: object, ndim: int) -> tuple[int, ...]:
    message = "size must be an integer or a sequence of integers"
    try:
        scalar = as_index(size, message)
    except TypeError:
        if isinstance(size, (str, bytes)) or not isinstance(size, Sequence):
            raise TypeError(message) from None
        entries = tuple(size)
        if len(entries) != ndim:
            raise ValueError("size sequence must have one entry per array dimension") from None
        values = tuple(
            as_index(entry, "size entries must be integers, not booleans") for entry in entries
        )
    else:
        values = (scalar,) * ndim
    if any(v <= 0 for v in values):
        raise ValueError("size entries must be positive integers")
    return values


def _window(size: object, footprint: object, origin: object, ndim: int):
    if footprint is None:
        shape = _sizes(3 if size is None else size, ndim)
        flat = None
        count = 1
        for length in shape:
            count *= length
    else:
        if size is not None:
            raise ValueError("pass either size or footprint, not both")
        if np.ma.isMaskedArray(footprint):
            raise TypeError("footprint must not be a masked array")
        entries = np.asarray(footprint)
        if entries.dtype.kind not in "biuf":
            raise TypeError("footprint must have a boolean or real numeric dtype")
        if entries.dtype.kind == "f" and not np.isfinite(entries).all():
            raise ValueError("footprint entries must be finite")
        selected = entries != 0
        if selected.ndim != ndim:
            raise ValueError("footprint must have the same rank as the array")
        if selected.size == 0:
            raise ValueError("footprint axes must be nonempty")
        count = int(np.count_nonzero(selected))
        if count == 0:
            raise ValueError("footprint must select at least one element")
        shape = tuple(int(n) for n in selected.shape)
        flat = selected.ravel().tolist()
    if np.ndim(origin) == 0:
        origins = (as_index(origin, "origin must be an integer or a sequence"),) * ndim
    else:
        if isinstance(origin, np.ndarray):
            origin = origin.tolist()
        origins = tuple(
            as_index(v, "origin entries must be integers, not booleans") for v in origin
        )
        if len(origins) != ndim:
            raise ValueError("origin sequence must have one entry per array dimension")
    for length, shift in zip(shape, origins):
        if not -(length // 2) <= shift <= (length - 1) // 2:
            raise ValueError("origin must satisfy -(size // 2) <= origin <= (size - 1) // 2")
    return shape, flat, origins, count


def _modes(mode: object, ndim: int) -> tuple[str, ...]:
    if isinstance(mode, str):
        values = (mode,) * ndim
    else:
        if not isinstance(mode, Sequence):
            raise TypeError("mode must be a string or a sequence of strings")
        values = tuple(mode)
        if len(values) != ndim:
            raise ValueError("mode sequence must have one entry per array dimension")
        if any(not isinstance(v, str) for v in values):
            raise TypeError("mode entries must be strings")
    if any(v not in MODES for v in values):
        raise ValueError(f"mode must use only {MODES}")
    return values


def validate(
    array: object,
    size: object,
    mode: object,
    cval: object,
    *,
    min_count: object,
    ddof: object = 0,
    footprint: object = None,
    origin: object = 0,
) -> Arguments:
    """Validate public arguments and return the native call's inputs."""
    value = check_array(array)
    shape, flat, origins, count = _window(size, footprint, origin, value.ndim)
    modes = _modes(mode, value.ndim)
    if isinstance(cval, (bool, np.bool_)) or not isinstance(cval, numbers.Real):
        raise TypeError("cval must be a non-boolean real scalar")
    cast_cval = float(value.dtype.type(cval))
    minimum = as_index(min_count, "min_count must be an integer, not a boolean")
    volume = 1
    for length in shape:
        volume *= length
        if volume > _INDEX_MAX:
            raise OverflowError("window volume exceeds the native index range")
    if minimum < 1 or minimum > count:
        raise ValueError("min_count must be between 1 and the number of window elements")
    dof = as_index(ddof, "ddof must be an integer, not a boolean")
    if dof < 0:
        raise ValueError("ddof must be nonnegative")
    if dof > _INDEX_MAX:
        raise OverflowError("ddof exceeds the native index range")
    if not value.flags.c_contiguous or type(value) is not np.ndarray:
        value = np.require(value, dtype=value.dtype, requirements=("C", "A", "O", "W"))
    return Arguments(
        array=value,
        size=shape,
        footprint=flat,
        origin=origins,
        mode=modes,
        cval=cast_cval,
        min_count=minimum,
        ddof=dof,
        count=count,
    )


def check_method(method: object, allowed: tuple[str, ...]) -> str:
    if not isinstance(method, str) or method not in allowed:
        raise ValueError(f"method must be one of {allowed}")
    return method


def check_flag(value: object, name: str) -> bool:
    if not isinstance(value, (bool, np.bool_)):
        raise TypeError(f"{name} must be a boolean")
    return bool(value)
