"""Exact rolling means (kind mean_rolling, method="boxcar") on the GPU
against the oracle's exact sums: bit for bit, every mode, origin and policy,
NaN / infinity counts, signed zeros, subnormals, and value ranges wide enough
to send tiles to the full-width kernel (src/boxcar.rs, src/exact_sum.rs;
tests/test_rolling_mean.py)."""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu

MODES = ("reflect", "constant", "nearest", "mirror", "wrap")


def _gpu(array, size, origin, mode, cval, omit, ignore_inf, min_count):
    from ndfiltrs_gb300 import _core

    with _core.Plan(array.shape, array.dtype, "mean_rolling", size, origin=origin, mode=mode, cval=cval,
                    omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count) as plan:
        return plan.run_host(np.ascontiguousarray(array)), plan.algorithm


def _values(shape, dtype, seed, wide=False):
    rng = np.random.default_rng(seed)
    if wide:
        # Magnitudes across the type's whole range: tiles need the full width.
        low, high = (-44, 37) if dtype == np.float32 else (-320, 300)
        values = rng.normal(size=shape) * 10.0 ** rng.integers(low, high, size=shape)
    else:
        values = 1000 + rng.normal(size=shape) * 10
    values = values.astype(dtype)
    special = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, np.finfo(dtype).tiny / 8], dtype=dtype)
    chosen = rng.random(shape) < 0.03
    values[chosen] = rng.choice(special, size=int(chosen.sum()))
    return values


KERNELS = {"band": "boxcar_band", "boxcar": "boxcar_tile"}


@pytest.fixture(params=sorted(KERNELS))
def kernel(request, gpu):
    """Pin the band or the tiled kernel for the test."""
    from ndfiltrs_gb300 import _core

    _core.pin_kernel(request.param)
    yield KERNELS[request.param]
    _core.pin_kernel(None)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", MODES)
def test_boxcar_matches_oracle(gpu, oracle, kernel, dtype, mode) -> None:
    for shape, size, origin in (((70, 90), (5, 7), (1, -2)), ((40, 33), (9, 4), (-4, 1)),
                                ((300,), (11,), (3,)), ((1, 500), (1, 31), (0, 0)),
                                ((6, 9, 8), (3, 2, 5), (0, 0, -1))):
        values = _values(shape, dtype, seed=len(shape) * 7 + size[0])
        volume = int(np.prod(size))
        for omit, ignore_inf, min_count in ((False, False, 1), (True, False, 1), (True, True, volume // 2)):
            for cval in (0.25, np.nan):
                args = (values, size, origin, [mode] * len(shape), cval, omit, ignore_inf, min_count)
                actual, algorithm = _gpu(*args)
                expected = oracle.window_filter(values, "mean_rolling", size, origin=origin, mode=mode,
                                                cval=cval, omit_nan=omit, ignore_inf=ignore_inf,
                                                min_count=min_count)
                np.testing.assert_array_equal(bits(actual), bits(expected),
                                              err_msg=str((shape, size, omit, cval, algorithm)))
                assert algorithm == ("boxcar_direct" if len(shape) == 3 else kernel)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_boxcar_wide_ranges_use_the_full_width_kernel(gpu, oracle, kernel, dtype) -> None:
    """Values from subnormals to near the overflow threshold in one tile or
    band: those go to a wider pass (bands) and then to the full-width
    kernel; results stay exact. A second array mixes narrow and wide
    regions."""
    wide = _values((64, 80), dtype, seed=3, wide=True)
    mixed = _values((130, 600), dtype, seed=4)
    mixed[100:, 520:] = _values((30, 80), dtype, seed=5, wide=True)
    for values in (wide, mixed):
        for omit in (False, True):
            actual, algorithm = _gpu(values, (7, 5), (0, 0), ["reflect", "wrap"], 0.0, omit, False, 1)
            expected = oracle.window_filter(values, "mean_rolling", (7, 5), mode=("reflect", "wrap"),
                                            omit_nan=omit)
            assert algorithm == kernel
            np.testing.assert_array_equal(bits(actual), bits(expected))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_boxcar_wide_windows(gpu, oracle, kernel, dtype) -> None:
    """Windows of 33 x 65 and 129 x 129 over images a few bands wide and
    tall, every mode, with the band height cut short at the bottom."""
    values = _values((700, 611), dtype, seed=9)
    for size, origin, mode in (((33, 65), (-3, 7), "reflect"), ((129, 129), (0, 0), "nearest"),
                               ((65, 17), (5, -8), "wrap"), ((17, 129), (0, 60), "constant"),
                               ((129, 3), (-64, 0), "mirror")):
        for omit, min_count in ((False, 1), (True, 100)):
            actual, algorithm = _gpu(values, size, origin, [mode] * 2, -1.5, omit, True, min_count)
            expected = oracle.window_filter(values, "mean_rolling", size, origin=origin, mode=mode,
                                            cval=-1.5, omit_nan=omit, ignore_inf=True,
                                            min_count=min_count)
            # A tile too large for shared memory leaves the band kernel.
            assert algorithm in (kernel, "boxcar_band")
            np.testing.assert_array_equal(bits(actual), bits(expected), err_msg=str((size, mode, omit)))


def test_boxcar_rounds_once_and_public_api(gpu, oracle) -> None:
    """tests/test_rolling_mean.py:118-137 through the public functions, plus
    large windows (histogram-sized boxes) on a sky-like image."""
    import ndfiltrs_gb300 as nf

    for dtype in (np.float32, np.float64):
        for odd_lower in (False, True):
            for direction in (-1, 0, 1):
                lower = dtype(1)
                if odd_lower:
                    lower = np.nextafter(lower, dtype(np.inf))
                upper = np.nextafter(lower, dtype(np.inf))
                tiny = np.nextafter(dtype(0), dtype(1))
                array = np.array([2 * lower, 2 * upper, direction * tiny, 0], dtype=dtype)
                expected = upper if direction > 0 or (direction == 0 and odd_lower) else lower
                actual = nf.mean_filter(array, 4, mode="wrap", method="boxcar")
                np.testing.assert_array_equal(actual, np.full(4, expected, dtype=dtype))
    rng = np.random.default_rng(9)
    sky = (500 + rng.normal(size=(200, 230)) * 22).astype(np.float32)
    sky[:, 17] = np.nan
    for size in ((65, 65), (31, 51)):
        actual = nf.nanmean_filter(sky, size, mode="nearest", method="boxcar")
        expected = oracle.window_filter(sky, "mean_rolling", size, mode="nearest", omit_nan=True)
        np.testing.assert_array_equal(bits(actual), bits(expected))
