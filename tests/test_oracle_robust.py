"""Pin the oracle's robust family to the reference's literal tests.

MAD, sigma clipping, the mode estimators and the biweight location / scale
(RobustReduction::finish, src/robust.rs:244-299; src/location.rs). Each
expectation restates a literal of the reference's Rust unit tests, cited per
test (ysBach/ndfiltrs v0.2.0). The biweight and mode references come from
astropy / astroimred / SExtractor and the reference checks them within
4 * eps relative (src/location.rs:281-288); the same tolerance applies here.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

MAX = np.finfo(np.float64).max
TINY = float(np.array([1], np.uint64).view(np.float64)[0])
NAN, INF = math.nan, math.inf


def _close(actual: float, expected: float) -> None:
    assert abs(actual - expected) <= 4 * np.finfo(np.float64).eps * abs(expected), (actual, expected)


def _modes(oracle, values):
    return [oracle.robust_values("mode", values, estimator=e, pearson=2.5 if e == "sex" else 3.0)
            for e in ("mmm", "iraf", "sex")]


A = [3.0, -1.5, 2.25, 8.0, 0.5, 1.75, 40.0, -6.0, 2.0, 1.0, 4.5]
B = [10.0, 11.0, 12.0, 13.0, 50.0, 9.5, 10.5, 11.5]


def test_modes_match_references(oracle) -> None:
    # src/location.rs:296-314
    cases = [
        (A, [-4.090909090909092, -4.090909090909092, -2.5681818181818183]),
        (B, [1.875, 1.875, 11.25]),
        ([0.0, 0.0, 0.0, 0.0, 1.0, 100.0], [-33.666666666666664, -33.666666666666664, 0.0]),
        ([-100.0, 1.0, 2.0, 3.0, 4.0], [42.0, -18.0, 2.0]),
    ]
    for values, expected in cases:
        for actual, want in zip(_modes(oracle, values), expected):
            _close(actual, want)


def test_mode_literals_empty_and_single(oracle) -> None:
    # src/location.rs:316-335
    assert _modes(oracle, [0.0, 1.0, 5.0]) == [-1.0, -1.0, 1.0]
    assert _modes(oracle, [-2.0, 0.0, 5.0])[2] == 0.0
    assert _modes(oracle, [1.0, 2.0, 3.0, 3.5])[2] == 2.6875
    assert _modes(oracle, [10.0] * 6 + [0.0, 0.0, -50.0])[2] == 10.0
    assert all(math.isnan(v) for v in _modes(oracle, []))
    assert _modes(oracle, [7.5]) == [7.5] * 3
    assert _modes(oracle, [MAX] * 4) == [MAX] * 3


def _loc(oracle, values, c):
    return oracle.robust_values("biweight_location", values, parameter=c)


def _scale(oracle, values, c, modify):
    return oracle.robust_values("biweight_scale", values, parameter=c, modify_sample_size=modify)


def test_biweight_matches_astropy(oracle) -> None:
    # src/location.rs:337-349
    _close(_loc(oracle, A, 6.0), 1.9602591329467531)
    _close(_loc(oracle, A, 4.0), 1.8351324381177168)
    _close(_scale(oracle, A, 9.0, False), 3.281179906799965)
    _close(_scale(oracle, A, 9.0, True), 3.128482289718106)
    _close(_scale(oracle, A, 3.0, True), 1.7300121556223182)
    _close(_loc(oracle, B, 6.0), 11.074571936132376)
    _close(_loc(oracle, B, 4.0), 11.079463959276655)
    _close(_scale(oracle, B, 9.0, False), 1.252142592975011)
    _close(_scale(oracle, B, 9.0, True), 1.1712721455748067)
    _close(_scale(oracle, B, 3.0, True), 1.8786667369052221)


def test_biweight_empty_single_zero_mad_and_symmetry(oracle) -> None:
    # src/location.rs:351-374
    assert math.isnan(_loc(oracle, [], 6.0)) and math.isnan(_scale(oracle, [], 9.0, False))
    assert _loc(oracle, [-3.5], 6.0) == -3.5 and _scale(oracle, [-3.5], 9.0, False) == 0.0
    assert _loc(oracle, [2.0, 2.0, 2.0, 9.0, -40.0], 6.0) == 2.0
    assert _scale(oracle, [2.0, 2.0, 2.0, 9.0, -40.0], 9.0, True) == 0.0
    assert abs(_loc(oracle, [5.0, 1.0, 9.0, 4.0, 6.0, 2.0, 8.0], 6.0) - 5.0) <= 4 * 2.220446049250313e-16 * 5
    assert _loc(oracle, [-1.0, 0.0, 1.0], 1.0) == 0.0
    expected = math.sqrt(3.0 * 2.0 * 0.25 * 0.75**4) / 0.625 * 2.0
    _close(_scale(oracle, [-1.0, 0.0, 1.0], 2.0, False), expected)


def test_biweight_large_magnitudes(oracle) -> None:
    # src/location.rs:376-402
    big = [v * 1e300 for v in A]
    _close(_loc(oracle, big, 6.0), 1.9602591329467533e300)
    _close(_scale(oracle, big, 9.0, False), 3.281179906799965e300)
    extremes = [-MAX, -MAX, 0.0, MAX, MAX]
    assert _loc(oracle, extremes, 6.0) == 0.0
    down, up = 2.0**-600, 2.0**600
    for values in (extremes, [-MAX, 0.5 * MAX, 0.75 * MAX, MAX, MAX]):
        small = [v * down for v in values]
        assert _loc(oracle, values, 6.0) == _loc(oracle, small, 6.0) * up
        for modify in (False, True):
            spread = _scale(oracle, values, 9.0, modify)
            assert math.isfinite(spread) and spread > 0
            assert spread == _scale(oracle, small, 9.0, modify) * up


def test_mode_and_biweight_follow_sample_policies(oracle) -> None:
    # src/robust.rs:812-878
    skewed = [1.0, 2.0, NAN, 3.0, 10.0]
    mode = lambda e, **kw: oracle.robust_values("mode", skewed, omit_nan=True, estimator=e,
                                                pearson=2.5 if e == "sex" else 3.0, **kw)
    assert mode("sex") == 2.5 and mode("mmm") == -0.5 and mode("iraf") == -0.5
    assert math.isnan(oracle.robust_values("mode", skewed, estimator="mmm", pearson=3.0))
    assert math.isnan(oracle.robust_values("mode", [1.0, INF], omit_nan=True, estimator="mmm", pearson=3.0))
    assert oracle.robust_values("biweight_location", [1.0, 2.0, 3.0, NAN], omit_nan=True, parameter=6.0) == 2.0
    assert math.isnan(oracle.robust_values("biweight_scale", [1.0, 2.0, -INF], omit_nan=True, parameter=9.0))
    clipped_mode = oracle.robust_values("sigma_mode", skewed, sigma_lower=10.0, sigma_upper=10.0, maxiters=1,
                                        estimator="mmm", pearson=3.0)
    assert clipped_mode == -0.5


def test_percentile_literals(oracle) -> None:
    # src/robust.rs:880-905, 907-921
    for q, expected in ((0.0, 1.0), (25.0, 2.5), (50.0, 4.0), (100.0, 9.0)):
        assert oracle.robust_values("percentile", [9.0, 1.0, 4.0], parameter=q) == expected
    omit = dict(omit_nan=True, ignore_inf=True, min_count=2, parameter=50.0)
    assert oracle.robust_values("percentile", [1.0, NAN, 3.0, INF], **omit) == 2.0
    assert math.isnan(oracle.robust_values("percentile", [1.0, NAN, INF], **omit))
    # src/robust.rs:1077-1088
    assert oracle.robust_values("percentile", [-TINY, 2 * TINY, NAN], omit_nan=True, parameter=50.0) == 0.0


def test_mad_literals(oracle) -> None:
    # src/robust.rs:923-952
    mad = lambda values, scale, **kw: oracle.robust_values("mad", values, parameter=scale, **kw)
    assert mad([1.0, 2.0, 100.0], 2.0) == 2.0
    assert mad([1.0, 2.0, INF], 2.0) == 2.0
    assert math.isnan(mad([1.0, INF, INF], 2.0))
    assert mad([-MAX, 0.5 * MAX, MAX], 0.25) == MAX * 0.125
    assert mad([-TINY, 0.0, TINY], MAX) == TINY * MAX
    # src/robust.rs:1090-1110
    assert mad([0.0, TINY, NAN], 2.0, omit_nan=True) == TINY
    assert mad([0.0, TINY, 2 * TINY, 4 * TINY], 2.0, omit_nan=True) == 2 * TINY
    assert mad([-MAX, -TINY, 0.0, MAX], 2.0, omit_nan=True) == MAX


def test_clipping_literals(oracle) -> None:
    # src/robust.rs:954-960
    values = [0.0, 0.0, 1.0, 2.0, 10.0, NAN, INF]
    clip = lambda maxiters: oracle.robust_values("sigma_mean", values, sigma_lower=1.0, sigma_upper=1.0,
                                                 maxiters=maxiters)
    assert clip(0) == 2.6 and clip(1) == 0.75 and clip(None) == 0.0
    # src/robust.rs:962-985
    mad_median = dict(sigma_lower=3.0, sigma_upper=3.0, maxiters=None, spread="mad")
    assert oracle.robust_values("sigma_median", [0.0, 0.0, 9.0], **mad_median) == 0.0
    assert math.isnan(oracle.robust_values("sigma_median", [0.0, 0.0, 9.0], min_count=3, **mad_median))
    # src/robust.rs:987-1021
    one = dict(maxiters=1, spread="mad")
    assert oracle.robust_values("sigma_mean", [0.0, 1.0, 2.0, 3.0, 4.5], sigma_lower=2.0, sigma_upper=2.0,
                                **one) == 2.1
    assert oracle.robust_values("sigma_mean", [-MAX, 0.0, MAX], sigma_lower=0.5, sigma_upper=0.5, **one) == 0.0
    # src/robust.rs:1112-1125
    assert oracle.robust_values("sigma_mean", [0.0, TINY, TINY], maxiters=None, min_count=3) == TINY
    # src/robust.rs:1127-1143
    assert oracle.robust_values("sigma_mean", [-MAX, -MAX, MAX], sigma_lower=1.5, sigma_upper=1.5,
                                maxiters=1) == -MAX


def test_robust_filter_geometry(oracle) -> None:
    # src/robust.rs:1145-1165 (reflect, size 3, q = 25) and canonical NaN
    # (src/robust.rs:1023-1053).
    out = oracle.robust_filter(np.array([1.0, 5.0, 9.0]), "percentile", 3, parameter=25.0)
    assert out.tolist() == [1.0, 3.0, 7.0]
    payload = np.array([0xFFF8000000000001], np.uint64).view(np.float64)
    for kind, kw in (("percentile", dict(parameter=50.0)), ("mad", dict(parameter=0.0)),
                     ("sigma_mean", dict(maxiters=None, sigma_lower=1.0, sigma_upper=1.0))):
        got = oracle.robust_filter(payload, kind, 1, **kw)
        assert got.view(np.uint64)[0] == 0x7FF8000000000000, kind
    with pytest.raises(oracle.OracleError):
        oracle.robust_filter(np.zeros(5), "mad", 3, omit_nan=True, min_count=4)
