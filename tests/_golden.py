"""Helpers to replay the committed golden vectors (tests/golden/golden_v1.*)."""

from __future__ import annotations

import numpy as np

from tests.conftest import bits


def case_kind(case: dict) -> str:
    family = case["family"]
    if family in ("median", "footprint_median", "padding"):
        return "median"
    return case["kind"]


def unpack(case: dict, arrays: dict):
    index = case["index"]
    array = arrays[f"in{index}"]
    expected = arrays[f"out{index}"]
    footprint = arrays[case["footprint"]] if case.get("footprint") else None
    size = case.get("size")
    if footprint is not None:
        size = list(footprint.shape)
    return array, expected, footprint, size


def statistic_rtol(dtype, volume: int) -> float:
    """The reference's rounding envelope for var/std (tests/test_statistics.py:59-72)."""
    operations = 12 * volume + 8
    unit64 = np.finfo(np.float64).eps / 2
    gamma = operations * unit64 / (1 - operations * unit64)
    return gamma + float(np.finfo(dtype).eps)


def assert_matches(actual: np.ndarray, expected: np.ndarray, case: dict, *, exact_moments: bool) -> None:
    assert actual.shape == expected.shape and actual.dtype == expected.dtype
    kind = case_kind(case)
    canonical = 0x7FC00000 if actual.dtype == np.float32 else 0x7FF8000000000000
    np.testing.assert_array_equal(np.isnan(actual), np.isnan(expected), err_msg=str(case))
    np.testing.assert_array_equal(bits(actual[np.isnan(actual)]), canonical, err_msg=str(case))
    if kind in ("var", "std"):
        np.testing.assert_array_equal(np.isposinf(actual), np.isposinf(expected))
        volume = int(np.prod(case["size"])) if case.get("size") else 9
        np.testing.assert_allclose(
            actual, expected, rtol=statistic_rtol(actual.dtype, volume), atol=0, err_msg=str(case)
        )
        return
    if kind == "mean" and not exact_moments:
        np.testing.assert_allclose(
            actual, expected, rtol=4 * float(np.finfo(actual.dtype).eps), atol=0, err_msg=str(case)
        )
        return
    np.testing.assert_array_equal(bits(actual), bits(expected), err_msg=str(case))


def native_kinds(case: dict, footprint) -> list[str]:
    kind = case_kind(case)
    if kind == "median":
        kinds = ["median", "median_network"]
        if footprint is None:
            kinds.append("median_histogram")
        return kinds
    if kind == "rank" and footprint is None:
        return ["rank", "rank_histogram"]
    return [kind]
