"""Generate the committed golden vectors under ``tests/golden/``.

The expected outputs come from the reference project's own independent
oracles, imported from a checkout of ysBach/ndfiltrs v0.2.0:

* ``tests/_reference.py`` (``median_filter_reference``, ``_map_index``,
  ``_median``): literal N-D median with the reducers midpoint contract;
* ``tests/_statistics_reference.py`` (``statistics_filter_reference``):
  exact rational variance, Decimal square root, signed-zero extrema;
* ``tests/_mean_reference.py`` (``mean_filter_reference``): exact rational mean;
* SciPy ``ndimage`` and NumPy percentiles, exactly where the reference's tests
  use them as oracles (finite odd windows, dyadic percentiles).

The case families restate the reference's test matrices
(``tests/test_properties.py``, ``tests/test_median_network.py``,
``tests/test_statistics.py``, ``tests/test_mean.py``, ``tests/test_robust.py``,
``tests/test_boundaries.py``, ``tests/test_footprint.py``). Inputs are seeded
and small, so the fixture stays a few hundred KB.

Run (needs the reference checkout; it is not needed to use the fixtures):

    python tests/golden/make_golden.py --reference /path/to/ndfiltrs
"""

from __future__ import annotations

import argparse
import json
import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
MODES = ("reflect", "constant", "nearest", "mirror", "wrap")


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument(
        "--reference",
        default=os.environ.get("NDFILTRS_REFERENCE"),
        help="checkout of the reference project (or set NDFILTRS_REFERENCE)",
    )
    parser.add_argument("--output", default=str(HERE / "golden_v1"))
    args = parser.parse_args()
    if not args.reference:
        parser.error("--reference (or NDFILTRS_REFERENCE) is required")
    sys.path.insert(0, args.reference)
    from scipy import ndimage
    from tests._mean_reference import mean_filter_reference
    from tests._reference import _map_index, _median, median_filter_reference
    from tests._statistics_reference import statistics_filter_reference

    cases: list[dict] = []
    arrays: dict[str, np.ndarray] = {}

    def add(family: str, array: np.ndarray, expected: np.ndarray, **params) -> None:
        index = len(cases)
        arrays[f"in{index}"] = np.ascontiguousarray(array)
        arrays[f"out{index}"] = np.ascontiguousarray(expected)
        if "footprint" in params and params["footprint"] is not None:
            arrays[f"fp{index}"] = np.asarray(params.pop("footprint"), dtype=bool)
            params["footprint"] = f"fp{index}"
        cases.append({"family": family, "index": index, **params})

    # A. Random small N-D medians (tests/test_properties.py:11-65).
    rng = np.random.default_rng(20261203)
    for _ in range(90):
        rank = int(rng.integers(1, 4))
        shape = tuple(int(v) for v in rng.integers(1, 6, size=rank))
        size = tuple(int(v) for v in rng.choice([1, 2, 3, 4, 5], size=rank))
        mode = tuple(str(m) for m in rng.choice(MODES, size=rank))
        dtype = np.float32 if rng.integers(0, 2) else np.float64
        values = rng.choice(
            [-np.inf, -3.5, -0.0, 0.0, 2.25, np.inf, np.nan, 1.0, 7.0], size=shape
        ).astype(dtype)
        omit = bool(rng.integers(0, 2))
        ignore_inf = bool(rng.integers(0, 2)) and omit
        volume = int(np.prod(size))
        min_count = int(rng.integers(1, volume + 1)) if omit else 1
        cval = float(dtype(rng.choice([-np.inf, -1.25, -0.0, 0.0, 4.0, np.inf, np.nan])))
        expected = median_filter_reference(
            values, size, mode, cval=cval, omit_nan=omit, ignore_inf=ignore_inf,
            min_count=min_count,
        )
        add("median", values, expected, size=list(size), mode=list(mode), origin=[0] * rank,
            cval=cval, omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count)

    # B. Literal sorted footprints with shifted origins
    #    (tests/test_median_network.py:48-118).
    geometries = [
        ((17,), (4,), (-2,)),
        ((7, 9), (3, 4), (1, -2)),
        ((4, 5, 7), (2, 3, 2), (-1, 0, 0)),
    ]
    for dtype in (np.float32, np.float64):
        for mode in MODES:
            for policy in ("plain", "omit", "finite", "minimum"):
                for shape, size, origin in geometries:
                    values = np.random.default_rng(712).normal(size=shape).astype(dtype)
                    special = [np.nan, np.inf, -np.inf, -0.0, 0.0,
                               np.finfo(dtype).max, -np.finfo(dtype).max]
                    values.flat[::7] = np.resize(np.asarray(special, dtype=dtype),
                                                 values.flat[::7].size)
                    footprint = np.indices(size).sum(axis=0) % 3 != 0
                    taps = np.argwhere(footprint)
                    omit = policy != "plain"
                    ignore_inf = policy == "finite"
                    min_count = len(taps) if policy == "minimum" else 1
                    cval = float(dtype(-0.0))
                    expected = np.empty_like(values)
                    for center in np.ndindex(shape):
                        samples = []
                        for tap in taps:
                            mapped = [
                                _map_index(c + int(k) - n // 2 - s, length, mode)
                                for c, k, n, s, length in zip(center, tap, size, origin, shape)
                            ]
                            value = float(cval if None in mapped else values[tuple(mapped)])
                            if (omit and math.isnan(value)) or (ignore_inf and math.isinf(value)):
                                continue
                            samples.append(value)
                        expected[center] = (
                            np.nan
                            if len(samples) < min_count or any(map(math.isnan, samples))
                            else _median(samples)
                        )
                    add("footprint_median", values, expected, footprint=footprint,
                        mode=[mode] * len(shape), origin=list(origin), cval=cval,
                        omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count)

    # C. Padding transitions with NaN payloads and signed zeros
    #    (tests/test_median_network.py:15-45).
    for dtype in (np.float32, np.float64):
        for count in (13, 17, 25, 33, 49, 65):
            for ignore_inf in (None, False, True):
                values = np.random.default_rng(129).normal(size=5 * count).astype(dtype)
                bits = np.uint32 if dtype is np.float32 else np.uint64
                payload = 0xFFC01234 if dtype is np.float32 else 0xFFF8000000001234
                values[count // 3 : 2 * count // 3] = np.array([payload], dtype=bits).view(dtype)[0]
                values[count + 2] = np.inf
                values[2 * count - 3] = -np.inf
                values[3 * count :] = np.resize(np.array([-0.0, 0.0], dtype=dtype), 2 * count)
                expected = median_filter_reference(
                    values, (count,), ("reflect",), cval=0.0,
                    omit_nan=ignore_inf is not None, ignore_inf=bool(ignore_inf), min_count=1,
                )
                add("padding", values, expected, size=[count], mode=["reflect"], origin=[0],
                    cval=0.0, omit_nan=ignore_inf is not None, ignore_inf=bool(ignore_inf),
                    min_count=1)

    # D. Extrema / variance / standard deviation with exact rational oracles
    #    (tests/test_statistics.py:108-125 and the NaN matrix).
    for dtype in (np.float32, np.float64):
        for shape in ((4,), (3, 4), (2, 1, 3), (2, 1, 2, 3)):
            for mode in MODES:
                array = ((np.arange(np.prod(shape)).reshape(shape) * 7) % 23 - 11).astype(dtype) / 4
                size = (5,) + (3,) * (len(shape) - 1)
                for statistic in ("min", "max", "var", "std"):
                    ddof = 1 if statistic in ("var", "std") else 0
                    expected = statistics_filter_reference(
                        array, size, (mode,) * array.ndim, statistic=statistic, cval=1.25,
                        ddof=ddof,
                    )
                    add("statistics", array, expected, kind=statistic, size=list(size),
                        mode=[mode] * len(shape), origin=[0] * len(shape), cval=1.25,
                        omit_nan=False, ignore_inf=False, min_count=1, parameter=ddof)
        # NaN-aware variants over values with NaN and infinities.
        for seed in range(6):
            r = np.random.default_rng(900 + seed)
            shape = (5, 6)
            array = (r.integers(-12, 13, size=shape) / 4).astype(dtype)
            array[r.random(shape) < 0.15] = np.nan
            array[r.random(shape) < 0.08] = np.inf
            array[r.random(shape) < 0.05] = -np.inf
            for statistic in ("min", "max", "var", "std"):
                for ignore_inf in (False, True):
                    ddof = 1 if statistic in ("var", "std") else 0
                    expected = statistics_filter_reference(
                        array, (3, 3), ("reflect", "wrap"), statistic=statistic, cval=0.5,
                        omit_nan=True, ignore_inf=ignore_inf, min_count=3, ddof=ddof,
                    )
                    add("statistics", array, expected, kind=statistic, size=[3, 3],
                        mode=["reflect", "wrap"], origin=[0, 0], cval=0.5, omit_nan=True,
                        ignore_inf=ignore_inf, min_count=3, parameter=ddof)

    # E. Means with exact rational sums (tests/test_mean.py:36-78).
    for dtype in (np.float32, np.float64):
        for mode in MODES:
            for shape in ((4,), (3, 4), (2, 1, 3), (2, 1, 2, 3)):
                size = (5,) + (3,) * (len(shape) - 1)
                volume = int(np.prod(size))
                array = (np.random.default_rng(20260906).integers(-32, 33, size=shape) * volume).astype(dtype)
                cval = 2.0 * volume
                expected = mean_filter_reference(array, size, (mode,) * array.ndim, cval=cval)
                add("mean", array, expected, kind="mean", size=list(size),
                    mode=[mode] * len(shape), origin=[0] * len(shape), cval=cval,
                    omit_nan=False, ignore_inf=False, min_count=1)
        array = np.array([[1, np.nan, np.inf], [-np.inf, 7, 11]], dtype=dtype)
        for ignore_inf in (False, True):
            for min_count in (1, 5, 15):
                for cval in (np.nan, np.inf, -np.inf, 2.0):
                    expected = mean_filter_reference(
                        array, (3, 5), ("constant", "mirror"), cval=cval, omit_nan=True,
                        ignore_inf=ignore_inf, min_count=min_count,
                    )
                    add("mean", array, expected, kind="mean", size=[3, 5],
                        mode=["constant", "mirror"], origin=[0, 0], cval=float(cval),
                        omit_nan=True, ignore_inf=ignore_inf, min_count=min_count)

    # F. Percentiles at dyadic q (tests/test_robust.py:23-38) and extreme ranks
    #    over footprints (tests/test_footprint.py:89-140).
    for dtype in (np.float32, np.float64):
        for mode in MODES:
            for q in (0.0, 12.5, 50.0, 87.5, 100.0):
                array = np.array([[3, -4, 8], [1, 12, -2]], dtype=dtype)
                expected = ndimage.generic_filter(
                    array, lambda v: np.percentile(v, q, method="linear"), size=(3, 5),
                    mode=mode, cval=1.25,
                )
                add("percentile", array, expected, kind="percentile", q=q, size=[3, 5],
                    mode=[mode, mode], origin=[0, 0], cval=1.25, omit_nan=False,
                    ignore_inf=False, min_count=1)
        fp = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], dtype=bool)
        for mode in MODES:
            values = np.random.default_rng(5).normal(size=(9, 11)).astype(dtype)
            count = int(fp.sum())
            for rank in (0, 1, count // 2, count - 1):
                expected = ndimage.rank_filter(values, rank, footprint=fp, mode=mode, cval=1.5,
                                               origin=(1, -1))
                add("rank", values, expected, kind="rank", parameter=rank, footprint=fp,
                    mode=[mode, mode], origin=[1, -1], cval=1.5, omit_nan=False,
                    ignore_inf=False, min_count=1)
            for q, rank in ((0.0, 0), (100.0, count - 1)):
                expected = ndimage.percentile_filter(values, q, footprint=fp, mode=mode,
                                                     cval=1.5, origin=(1, -1))
                add("percentile", values, expected, kind="percentile", q=q, footprint=fp,
                    mode=[mode, mode], origin=[1, -1], cval=1.5, omit_nan=False,
                    ignore_inf=False, min_count=1)

    # G. SciPy median on finite odd windows (tests/test_boundaries.py:8-15).
    for dtype in (np.float32, np.float64):
        for mode in MODES:
            values = np.arange(24, dtype=dtype).reshape(2, 3, 4)
            expected = ndimage.median_filter(values, size=(3, 1, 5), mode=mode, cval=-7.0)
            add("median", values, expected, size=[3, 1, 5], mode=[mode] * 3, origin=[0, 0, 0],
                cval=-7.0, omit_nan=False, ignore_inf=False, min_count=1)

    # H. Rank-5 mixed modes (tests/test_semantics.py:76-102).
    values = np.arange(48.0, dtype=np.float64).reshape(2, 2, 2, 2, 3)
    values[0, 1, 0, 1, 2] = np.nan
    size = (3, 3, 3, 3, 5)
    mode = ("reflect", "constant", "nearest", "mirror", "wrap")
    expected = median_filter_reference(values, size, mode, cval=-4.0, omit_nan=True,
                                       ignore_inf=False, min_count=7)
    add("median", values, expected, size=list(size), mode=list(mode), origin=[0] * 5,
        cval=-4.0, omit_nan=True, ignore_inf=False, min_count=7)

    out = Path(args.output)
    np.savez_compressed(out.with_suffix(".npz"), **arrays)
    out.with_suffix(".json").write_text(json.dumps({"version": 1, "cases": cases}, indent=0))
    print(f"wrote {len(cases)} cases to {out}.npz/.json")


if __name__ == "__main__":
    main()
