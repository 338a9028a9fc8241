"""The oracle's separable passes equal its direct window traversal.

WindowFilter::new (src/plan.rs:267-289) sends rectangular minimum / maximum
to van Herk passes (src/extrema.rs:124-437) and rolling means to exact
running sums (src/boxcar.rs:140-342). The oracle restates both, so the CPU
baseline times the reference's own algorithms; these tests check them bit for
bit against the oracle's direct traversal over the same case families as
the reference's tests (src/extrema.rs:627-790, src/boxcar.rs:348-418):
every short 1-D geometry, every origin tuple of small 2-D / 3-D windows,
random mixed geometry, empty arrays, and NaN payloads, signed zeros and
infinities in the samples and in cval.
"""

from __future__ import annotations

import itertools

import numpy as np
import pytest

from tests.conftest import bits

MODES = ["reflect", "constant", "nearest", "mirror", "wrap"]


def _values(rng: np.random.Generator, n: int, offset: int, dtype) -> np.ndarray:
    """Samples cycling through +0, -0, +inf, -inf, two NaN payloads, finite."""
    finite = (rng.integers(-20000, 20001, n) / 31.0).astype(dtype)
    out = np.empty(n, dtype)
    ut = np.uint32 if dtype == np.float32 else np.uint64
    nan_a = np.array([0x7FC00042 if dtype == np.float32 else 0x7FF8000000000042], ut).view(dtype)[0]
    nan_b = np.array([0xFFC00123 if dtype == np.float32 else 0xFFF8000000000123], ut).view(dtype)[0]
    special = [dtype(0.0), dtype(-0.0), dtype(np.inf), dtype(-np.inf), nan_a, nan_b]
    for i in range(n):
        k = (i + offset) % 8
        out[i] = special[k] if k < 6 else finite[i]
    return out


def _cvals(dtype):
    return [dtype(431 / 31.0), dtype(np.inf), dtype(-np.inf), dtype(np.nan)]


def _policies(volume: int):
    return [
        dict(omit_nan=False),
        dict(omit_nan=True, min_count=1),
        dict(omit_nan=True, min_count=volume),
        dict(omit_nan=True, ignore_inf=True, min_count=1),
        dict(omit_nan=True, ignore_inf=True, min_count=volume),
    ]


def _same(oracle, array, kind, **kw) -> None:
    fast = oracle.window_filter(array, kind, threads=2, **kw)
    slow = oracle.window_filter(array, kind, direct=True, threads=1, **kw)
    assert np.array_equal(bits(fast), bits(slow)), (kind, array.shape, kw)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extrema_every_short_line(oracle, dtype) -> None:
    rng = np.random.default_rng(7)
    case = 0
    for length in range(1, 6):
        for win in range(1, 7):
            for origin in range(-(win // 2), (win - 1) // 2 + 1):
                for mode in MODES:
                    for policy in _policies(win):
                        cval = _cvals(dtype)[case % 4]
                        x = _values(rng, length, case, dtype)
                        for kind in ("min", "max"):
                            _same(oracle, x, kind, size=win, origin=origin, mode=mode,
                                  cval=float(cval), **policy)
                        case += 1


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extrema_every_origin_tuple(oracle, dtype) -> None:
    rng = np.random.default_rng(11)
    case = 0
    for shape in [(1, 2), (1, 1, 2), (3, 4), (2, 3, 4)]:
        rank = len(shape)
        for win in range(1, 7 if len(shape) < 3 or max(shape) < 3 else 4):
            span = range(-(win // 2), (win - 1) // 2 + 1)
            for origin in itertools.product(span, repeat=rank):
                x = _values(rng, int(np.prod(shape)), case, dtype).reshape(shape)
                for mode in MODES:
                    policy = _policies(win**rank)[case % 5]
                    for kind in ("min", "max"):
                        _same(oracle, x, kind, size=win, origin=origin, mode=mode,
                              cval=float(_cvals(dtype)[case % 4]), **policy)
                    case += 1


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_extrema_random_mixed_geometry(oracle, dtype) -> None:
    rng = np.random.default_rng(13)
    for case in range(400):
        rank = 1 + case % 3
        shape = tuple(int(v) for v in rng.integers(1, 8, rank))
        size = tuple(int(v) for v in rng.integers(1, 7, rank))
        origin = tuple(int(rng.integers(-(s // 2), (s - 1) // 2 + 1)) for s in size)
        mode = tuple(MODES[int(v)] for v in rng.integers(0, 5, rank))
        x = _values(rng, int(np.prod(shape)), case, dtype).reshape(shape)
        policy = _policies(int(np.prod(size)))[case % 5]
        for kind in ("min", "max"):
            _same(oracle, x, kind, size=size, origin=origin, mode=mode,
                  cval=float(_cvals(dtype)[case % 4]), **policy)


def test_extrema_empty_arrays(oracle) -> None:
    for shape, size in [((0,), (3,)), ((0, 2), (4, 2)), ((1, 0, 2), (2, 3, 4))]:
        x = np.zeros(shape, np.float64)
        out = oracle.window_filter(x, "min", size=size, mode="constant", omit_nan=True,
                                   ignore_inf=True)
        assert out.shape == shape


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_rolling_mean_axis_passes(oracle, dtype) -> None:
    # The shapes, sizes and origins of src/boxcar.rs:348-418, every rotation
    # of the modes over the axes, three policies and three cvals.
    special = [np.nan, np.inf, -np.inf, -0.0, 1.0e20, -1.0e20]
    for shape in [(5,), (3, 5), (2, 3, 5), (2, 2, 3, 5)]:
        rank = len(shape)
        size = tuple(2 + a % 2 for a in range(rank))
        origin = tuple(-1 if s == 2 else 1 for s in size)
        n = int(np.prod(shape))
        x = np.array([special[i % 11] if i % 11 < 6 else i - 7.0 for i in range(n)],
                     dtype).reshape(shape)
        for shift in range(5):
            mode = tuple(MODES[(a + shift) % 5] for a in range(rank))
            for policy in [dict(omit_nan=False), dict(omit_nan=True, min_count=1),
                           dict(omit_nan=True, ignore_inf=True, min_count=2)]:
                for cval in (-0.0, 4.0, np.nan):
                    _same(oracle, x, "mean_rolling", size=size, origin=origin, mode=mode,
                          cval=cval, **policy)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_rolling_mean_wide_spans(oracle, dtype) -> None:
    # Spans from subnormals to near the largest finite value, cancellation
    # to exact zero, and windows long enough to carry across words.
    rng = np.random.default_rng(17)
    info = np.finfo(dtype)
    for case in range(60):
        rank = 1 + case % 2
        shape = tuple(int(v) for v in rng.integers(3, 12, rank))
        size = tuple(int(v) for v in rng.integers(1, 8, rank))
        origin = tuple(int(rng.integers(-(s // 2), (s - 1) // 2 + 1)) for s in size)
        mode = tuple(MODES[int(v)] for v in rng.integers(0, 5, rank))
        n = int(np.prod(shape))
        scale = [1.0, float(info.tiny), float(info.max) / 64, 1e-3][case % 4]
        x = (rng.standard_normal(n) * scale).astype(dtype)
        x[rng.integers(0, n, max(1, n // 5))] = dtype(info.smallest_subnormal)
        if case % 3 == 0:
            x[: n // 2] = -x[n // 2 : 2 * (n // 2)]
        x = x.reshape(shape)
        cval = [0.0, float(info.smallest_subnormal), -2.5, float(info.max) / 1e3][case % 4]
        policy = _policies(int(np.prod(size)))[case % 5]
        _same(oracle, x, "mean_rolling", size=size, origin=origin, mode=mode, cval=cval,
              **policy)


def test_separable_paths_are_the_default(oracle) -> None:
    # A 2-D 4-connected footprint keeps the direct path for min / max; the
    # rectangle takes the separable passes, with the same results.
    x = _values(np.random.default_rng(19), 48, 0, np.float64).reshape(6, 8)
    cross = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], bool)
    a = oracle.window_filter(x, "min", footprint=cross, omit_nan=True)
    b = oracle.window_filter(x, "min", footprint=cross, omit_nan=True, direct=True)
    assert np.array_equal(bits(a), bits(b))
    with pytest.raises(oracle.OracleError):
        oracle.window_filter(x, "mean_rolling", footprint=cross)
