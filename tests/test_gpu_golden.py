"""The CUDA library reproduces every committed golden vector (through the
package's native module, i.e. the C-ABI)."""

from __future__ import annotations

import pytest

from tests._golden import assert_matches, case_kind, native_kinds, unpack

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("moments", ["fp64", "fp32c"])
def test_gpu_reproduces_golden_vectors(gpu, golden_cases, moments, monkeypatch) -> None:
    from ndfiltrs_gb300 import _core

    monkeypatch.setenv("NDF_MOMENTS", moments)
    cases, arrays = golden_cases
    checked = 0
    for case in cases:
        array, expected, footprint, size = unpack(case, arrays)
        kind = case_kind(case)
        if moments == "fp32c" and kind not in ("mean", "var", "std"):
            continue
        for native in native_kinds(case, footprint):
            if native == "percentile":
                actual = _core.robust_filter(
                    array, size, footprint, case["origin"], case["mode"], case["cval"],
                    "percentile", case["q"], case["omit_nan"], case["ignore_inf"],
                    case["min_count"], 3.0, 3.0, 5, "median", "std",
                )
            else:
                actual = _core.window_filter(
                    array, native, size, footprint, case["origin"], case["mode"], case["cval"],
                    case["omit_nan"], case["ignore_inf"], case["min_count"], case.get("parameter", 0),
                )
            assert_matches(actual, expected, {**case, "kind": kind}, exact_moments=moments == "fp64")
            checked += 1
    assert checked > 100
