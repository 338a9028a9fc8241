"""Pin the CPU oracle to the reference's own known-answer tests.

Each test restates literal expectations from the reference's Rust unit tests
or Python contract tests (ysBach/ndfiltrs v0.2.0, cited per test). The oracle
is trusted as the parity checker of the CUDA library only because it passes
these and the golden vectors in test_oracle_golden.py.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = []


def test_boundary_literal_coordinates(oracle) -> None:
    # src/boundary.rs:77-118
    coordinates = [-5, -4, -3, -2, -1, 0, 1, 2, 3, 4, 5, 6, 7, 8]
    cases = {
        "reflect": [3, 3, 2, 1, 0, 0, 1, 2, 3, 3, 2, 1, 0, 0],
        "mirror": [1, 2, 3, 2, 1, 0, 1, 2, 3, 2, 1, 0, 1, 2],
        "nearest": [0, 0, 0, 0, 0, 0, 1, 2, 3, 3, 3, 3, 3, 3],
        "wrap": [3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0],
    }
    for mode, expected in cases.items():
        assert [oracle.map_index(c, 4, mode) for c in coordinates] == expected, mode


def test_constant_marks_only_outside(oracle) -> None:
    # src/boundary.rs:120-126
    assert [oracle.map_index(i, 2, "constant") for i in range(-2, 4)] == [None, None, 0, 1, None, None]


def test_length_two_axes(oracle) -> None:
    # src/boundary.rs:128-152
    coordinates = [-5, -4, -3, -2, -1, 0, 1, 2, 3, 4, 5, 6]
    cases = {
        "reflect": [0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1],
        "mirror": [1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0],
        "nearest": [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1],
        "wrap": [1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0],
    }
    for mode, expected in cases.items():
        assert [oracle.map_index(c, 2, mode) for c in coordinates] == expected


def test_singleton_and_many_periods(oracle) -> None:
    # src/boundary.rs:154-187
    for mode in ("reflect", "nearest", "mirror", "wrap"):
        for index in (-1_000_000, -1, 0, 1, 1_000_000):
            assert oracle.map_index(index, 1, mode) == 0
    assert oracle.map_index(1_000_000_003, 4, "reflect") == 3
    assert oracle.map_index(-1_000_000_003, 4, "mirror") == 1
    assert oracle.map_index(-1_000_000_003, 4, "wrap") == 1


def test_tap_order_with_footprint_and_origin(oracle) -> None:
    # src/window.rs:310-340: even footprint [1,0,1,1], anchor 2 + origin -1 = 1
    taps = oracle.window_taps((6,), (4,), footprint=np.array([1, 0, 1, 1]), origin=(-1,))
    assert taps[:, 0].tolist() == [-1, 1, 2]
    values = np.arange(6, dtype=np.float64)
    out = oracle.window_filter(
        values, "rank", footprint=np.array([1, 0, 1, 1]), origin=(-1,), mode="reflect", parameter=0
    )
    # samples at 2: [1, 3, 4]; at 5: [4, 5, 4]
    assert out[2] == 1.0 and out[5] == 4.0


def test_rectangular_constant_and_nearest_gather(oracle) -> None:
    # src/window.rs:297-308: 3x3 window over 0..8, modes (constant, nearest),
    # cval -1: at the corner the samples are [-1,-1,-1,0,0,1,3,3,4].
    values = np.arange(9, dtype=np.float64).reshape(3, 3)
    samples = np.array([-1, -1, -1, 0, 0, 1, 3, 3, 4], dtype=np.float64)
    for rank in range(9):
        out = oracle.window_filter(
            values, "rank", (3, 3), mode=("constant", "nearest"), cval=-1.0, parameter=rank
        )
        assert out[0, 0] == np.sort(samples)[rank]


def test_signed_zero_total_order(oracle) -> None:
    # src/reduction.rs:136-167
    def rank(values, r):
        a = np.array(values, dtype=np.float64)
        return oracle.window_filter(a, "rank", len(a), mode="wrap", parameter=r)[len(a) // 2]

    assert bits(np.array([rank([3.0, -0.0, 0.0, 1.0], 1)]))[0] == bits(np.array([0.0]))[0]
    beyond = oracle.window_filter(np.array([3.0, 1.0]), "rank", 2, mode="wrap", parameter=2)
    assert np.isnan(beyond).all()
    mn = oracle.window_filter(np.array([0.0, -0.0, 1.0]), "min", 3, mode="wrap")
    assert np.signbit(mn[1])
    mx = oracle.window_filter(np.array([-0.0, 0.0, -1.0]), "max", 3, mode="wrap")
    assert not np.signbit(mx[1]) and mx[1] == 0.0


def test_dispersion_counts_after_omission(oracle) -> None:
    # src/reduction.rs:169-185
    values = np.array([1.0, np.nan, np.inf, 3.0])
    kept = [1.0, 3.0]
    assert oracle.dispersion_valid(kept, 0, False) == 1.0
    assert oracle.dispersion_valid(kept, 1, True) == math.sqrt(2.0)
    assert math.isnan(oracle.dispersion_valid(kept, 2, True))
    out = oracle.window_filter(values, "var", 4, mode="wrap", omit_nan=True, ignore_inf=True, min_count=2)
    assert out[2] == 1.0


def test_propagate_and_omit_policies(oracle) -> None:
    # src/reduction.rs:187-212
    plain = oracle.window_filter(
        np.array([1.0, np.frombuffer(np.uint64(0x7FF0000000000001).tobytes(), np.float64)[0], 3.0]),
        "median",
        3,
        mode="wrap",
    )
    assert bits(plain)[1] == 0x7FF8000000000000
    omit = oracle.window_filter(
        np.array([1.0, np.nan, np.inf, 3.0]), "median", 4, mode="wrap", omit_nan=True,
        ignore_inf=True, min_count=2,
    )
    assert omit[2] == 2.0
    short = oracle.window_filter(
        np.array([1.0, np.nan, np.inf]), "median", 3, mode="wrap", omit_nan=True,
        ignore_inf=True, min_count=2,
    )
    assert bits(short)[1] == 0x7FF8000000000000


def test_reducer_contract(oracle) -> None:
    # src/reduction.rs:214-249 and tests/test_reducers_contract.py:8-48
    z = oracle.window_filter(np.array([0.0, -0.0, -0.0]), "median", 3, mode="wrap")
    assert np.signbit(z[1])
    big = np.finfo(np.float64).max
    prev = np.nextafter(big, 0.0)
    assert np.isfinite(oracle.midpoint(prev, big))
    assert math.isnan(oracle.midpoint(-np.inf, np.inf))
    assert bits(np.array([oracle.midpoint(-0.0, 0.0)]))[0] == 0
    upper = np.float32(np.nextafter(np.float32(1.0), np.float32(2.0)))
    values = np.array([1.0, upper], dtype=np.float32)
    out = oracle.window_filter(values, "median", 2, mode="wrap")
    expected = np.float32((1.0 + float(upper)) / 2.0)
    assert bits(out)[0] == bits(np.array([expected]))[0]
    for dtype in (np.float32, np.float64):
        maximum = np.finfo(dtype).max
        previous = np.nextafter(maximum, dtype(0), dtype=dtype)
        arr = np.asarray([maximum, previous, np.nan], dtype=dtype)
        got = oracle.window_filter(arr, "median", 3, mode="constant", cval=np.nan, omit_nan=True)
        assert np.isfinite(got[1]) and got[1] == dtype(previous + (maximum - previous) / dtype(2))
        for inf in (-np.inf, np.inf):
            arr = np.asarray([inf, inf, np.nan], dtype=dtype)
            got = oracle.window_filter(arr, "median", 3, mode="constant", cval=np.nan, omit_nan=True)
            assert got[1] == inf
        rep = np.asarray([2.0, 2.0, 4.0, 4.0, np.nan], dtype=dtype)
        got = oracle.window_filter(rep, "median", 5, mode="constant", cval=np.nan, omit_nan=True)
        assert got[2] == dtype(3.0)


def test_mean_literals(oracle) -> None:
    # src/mean.rs:119-149
    assert oracle.mean_valid([1e16, 1.0, -1e16]) == 1.0 / 3.0
    big = np.finfo(np.float64).max
    assert oracle.mean_valid([big] * 3) == big
    assert oracle.mean_valid([-big] * 4) == -big
    assert oracle.mean_valid([big, big, -big]) == big / 3.0
    assert oracle.mean_valid([big, big, -np.inf]) == -np.inf
    assert math.isnan(oracle.mean_valid([np.inf, -np.inf]))
    assert oracle.mean_valid([5e-324] * 3) == 5e-324
    out = oracle.window_filter(np.array([1.0, np.nan, 3.0]), "mean", 3, mode="nearest",
                               omit_nan=True, ignore_inf=True, min_count=2)
    assert out.tolist() == [1.0, 2.0, 3.0]


def test_dispersion_literals(oracle) -> None:
    # src/dispersion.rs:66-94
    assert oracle.dispersion_valid([1e16, 1e16 + 2.0, 1e16 + 4.0], 0, False) == 8.0 / 3.0
    assert oracle.dispersion_valid([1e16, 1e16 + 2.0], 0, False) == 1.0
    big = np.finfo(np.float64).max
    assert oracle.dispersion_valid([big] * 3, 0, False) == 0.0
    assert oracle.dispersion_valid([-big, big], 0, True) == big
    assert math.isinf(oracle.dispersion_valid([-big, big], 0, False))
    assert oracle.dispersion_valid([-1e-200, 1e-200], 0, True) == 1e-200
    assert oracle.dispersion_valid([-1e-200, 1e-200], 0, False) == 0.0
    assert oracle.dispersion_valid([1.0, 2.0, 3.0], 1, False) == 1.0
    for values in ([1.0], [np.inf, 1.0]):
        assert math.isnan(oracle.dispersion_valid(values, 1, True))


def test_percentile_interpolation_literals(oracle) -> None:
    # src/robust.rs:876-896 and :1042-1052
    big = np.finfo(np.float64).max
    assert oracle.interpolate(-big, big, 0.5) == 0.0
    assert oracle.interpolate(big, big, 0.75) == big
    assert oracle.interpolate(2.0, np.inf, 0.0) == 2.0
    assert oracle.interpolate(2.0, np.inf, 0.5) == np.inf
    assert oracle.interpolate(-np.inf, 2.0, 1.0) == 2.0
    assert math.isnan(oracle.interpolate(-np.inf, np.inf, 0.5))
    for q, expected in ((0.0, 1.0), (25.0, 2.5), (50.0, 4.0), (100.0, 9.0)):
        assert oracle.percentile([9.0, 1.0, 4.0], q) == expected
    assert bits(np.array([oracle.interpolate(-0.0, 0.0, 0.5)]))[0] == 0
    tiny = 5e-324
    out = oracle.window_filter(np.array([-tiny, 2 * tiny, np.nan]), "percentile", 3, mode="wrap",
                               omit_nan=True, q=50.0)
    assert out[1] == 0.0
    out = oracle.window_filter(np.array([1.0, 5.0, 9.0]), "percentile", 3, mode="reflect", q=25.0)
    assert out.tolist() == [1.0, 3.0, 7.0]


def test_percentile_omission(oracle) -> None:
    # src/robust.rs:898-913
    v = np.array([1.0, np.nan, 3.0, np.inf])
    out = oracle.window_filter(v, "percentile", 4, mode="wrap", omit_nan=True, ignore_inf=True,
                               min_count=2, q=50.0)
    assert out[2] == 2.0
    v = np.array([1.0, np.nan, np.inf])
    out = oracle.window_filter(v, "percentile", 3, mode="wrap", omit_nan=True, ignore_inf=True,
                               min_count=2, q=50.0)
    assert math.isnan(out[1])


@pytest.mark.parametrize("count", range(1, 13))
@pytest.mark.parametrize("omit", [False, True])
def test_zero_one_principle(oracle, count: int, omit: bool) -> None:
    # src/median_network.rs:267-307: every binary input of `count` taps.
    width = 1 << count
    columns = np.arange(width)
    planes = ((columns[None, :] >> np.arange(count)[:, None]) & 1).astype(np.float64)
    # Lay each column out as one window of a 1-D wrap array.
    for column in range(0, width, max(1, width // 64)):
        window = planes[:, column]
        arr = np.concatenate([window])
        out = oracle.window_filter(arr, "median_network", count, mode="wrap", omit_nan=omit,
                                   origin=-(count // 2))
        ones = int(window.sum())
        expected = 0.0 if 2 * ones < count else (0.5 if 2 * ones == count else 1.0)
        assert out[0] == expected, (count, column)


def test_histogram_select_in_word_equivalent(oracle) -> None:
    # src/histogram.rs:637-645 via results: rank filters over many ranks
    rng = np.random.default_rng(1)
    values = rng.integers(-4, 5, size=(40, 45)).astype(np.float64) / 4
    for rank in (0, 7, 24, 48):
        a = oracle.window_filter(values, "rank_histogram", (7, 7), mode="mirror", parameter=rank)
        b = oracle.window_filter(values, "rank", (7, 7), mode="mirror", parameter=rank)
        np.testing.assert_array_equal(bits(a), bits(b))


def test_histogram_rejects_oversized_support(oracle) -> None:
    # src/histogram.rs:802-810
    from oracle.oracle import OracleError

    with pytest.raises(OracleError):
        oracle.window_filter(np.zeros((1, 1)), "median_histogram", (70000, 70000))


# ---------------------------------------------------------------------------
# Exact boxcar mean (kind mean_rolling): src/boxcar.rs, src/exact_sum.rs.

def _round_exact(value, dtype):
    """The rational `value` rounded once to `dtype` (nearest, ties to even):
    the nearest of the float64-derived candidate and its two neighbours."""
    from fractions import Fraction

    if value == 0:
        return dtype(0)
    candidate = dtype(float(value))
    neighbours = [candidate, np.nextafter(candidate, dtype(-np.inf)), np.nextafter(candidate, dtype(np.inf))]
    ubits = np.uint32 if dtype == np.float32 else np.uint64
    return min((c for c in neighbours if np.isfinite(c)),
               key=lambda c: (abs(Fraction(float(c)) - value), int(np.array(c, dtype=dtype).view(ubits)) & 1))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("odd_lower", [False, True])
@pytest.mark.parametrize("direction", [-1, 0, 1])
def test_boxcar_mean_rounds_once_beside_midpoints(oracle, dtype, odd_lower, direction) -> None:
    """tests/test_rolling_mean.py:118-137: the mean (lower + upper) / 2 +
    direction * tiny / 4 rounds once, directly to the dtype."""
    lower = dtype(1)
    if odd_lower:
        lower = np.nextafter(lower, dtype(np.inf))
    upper = np.nextafter(lower, dtype(np.inf))
    tiny = np.nextafter(dtype(0), dtype(1))
    array = np.array([2 * lower, 2 * upper, direction * tiny, 0], dtype=dtype)
    expected = upper if direction > 0 or (direction == 0 and odd_lower) else lower
    out = oracle.window_filter(array, "mean_rolling", (4,), mode="wrap")
    np.testing.assert_array_equal(out, np.full(4, expected, dtype=dtype))


def test_boxcar_mean_matches_rational_reference(oracle) -> None:
    """Exact rational window means with NaN / inf counts, rounded once (the
    rule of tests/test_rolling_mean.py:49-85), over wide-range values."""
    import math
    from fractions import Fraction

    rng = np.random.default_rng(12)
    for trial in range(120):
        dtype = np.float32 if trial % 2 else np.float64
        n = int(rng.integers(3, 10))
        scale = 30 if dtype == np.float32 else 280
        arr = (rng.normal(size=n) * 10.0 ** rng.integers(-scale, scale, size=n)).astype(dtype)
        if trial % 3 == 0:
            arr[rng.integers(0, n)] = [np.nan, np.inf, -np.inf, -0.0][trial % 4]
        size = int(rng.integers(1, n + 1))
        omit, ignore_inf = bool(trial % 2), bool(trial % 5 == 0)
        out = oracle.window_filter(arr, "mean_rolling", (size,), mode="wrap", omit_nan=omit,
                                   ignore_inf=ignore_inf)
        for c in range(n):
            values = [float(arr[(c + k - size // 2) % n]) for k in range(size)]
            if omit:
                values = [v for v in values if not (math.isnan(v) or (ignore_inf and math.isinf(v)))]
            if not values or any(math.isnan(v) for v in values) or (math.inf in values and -math.inf in values):
                expected = dtype(np.nan)
            elif math.inf in values:
                expected = dtype(np.inf)
            elif -math.inf in values:
                expected = dtype(-np.inf)
            else:
                expected = _round_exact(sum(map(Fraction, values), Fraction()) / len(values), dtype)
            if np.isnan(expected):
                assert np.isnan(out[c])
            else:
                ubits = np.uint32 if dtype == np.float32 else np.uint64
                assert np.array(out[c]).view(ubits) == np.array(expected, dtype=dtype).view(ubits), \
                    (trial, c, out[c], expected)
