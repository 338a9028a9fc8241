"""The CPU oracle reproduces every committed golden vector.

The golden vectors were produced by the reference's own independent oracles
(tests/golden/make_golden.py). Passing them is what lets the oracle stand in
as the parity checker for the CUDA library on inputs too large to store.
"""

from __future__ import annotations

import numpy as np

from tests._golden import assert_matches, case_kind, native_kinds, unpack


def test_golden_families_present(golden_cases) -> None:
    cases, _ = golden_cases
    families = {case["family"] for case in cases}
    assert families >= {"median", "footprint_median", "padding", "statistics", "mean", "percentile", "rank"}
    assert len(cases) > 600


def test_oracle_reproduces_golden_vectors(oracle, golden_cases) -> None:
    cases, arrays = golden_cases
    for case in cases:
        array, expected, footprint, size = unpack(case, arrays)
        for kind in native_kinds(case, footprint):
            actual = oracle.window_filter(
                array,
                kind,
                size,
                footprint=footprint,
                origin=case["origin"],
                mode=case["mode"],
                cval=case["cval"],
                omit_nan=case["omit_nan"],
                ignore_inf=case["ignore_inf"],
                min_count=case["min_count"],
                parameter=case.get("parameter", 0),
                q=case.get("q", 50.0),
                threads=2,
            )
            assert_matches(actual, expected, {**case, "kind": case_kind(case)}, exact_moments=True)


def test_oracle_thread_count_invariance(oracle) -> None:
    # tests/test_parallel.py:48-89: outputs are bitwise identical for 1/2/4 workers.
    rng = np.random.default_rng(319)
    for dtype in (np.float32, np.float64):
        values = rng.normal(size=(17, 19)).astype(dtype)
        values[::5, ::4] = np.nan
        values[1::6, 2::7] = np.inf
        for kind in ("median", "median_network", "median_histogram", "mean", "var", "std", "min", "max"):
            outs = [
                oracle.window_filter(values, kind, (5, 3), mode=("mirror", "wrap"), omit_nan=True,
                                     threads=t).tobytes()
                for t in (1, 2, 4)
            ]
            assert len(set(outs)) == 1, kind
