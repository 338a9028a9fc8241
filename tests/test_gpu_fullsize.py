"""Parity at the benchmark configurations' full sizes.

The oracle is too slow for whole 4096^2 / 8192^2 images, so each full-size
GPU result is checked (a) bit for bit against the oracle on row strips: the
top and bottom edges and random interior strips, each filtered by the oracle
from a crop with the window's vertical halo (so every compared row sees the
same samples as in the full image), and (b) through size-independent
properties: min <= median <= max, percentiles monotone in q, ranks sorted in
k, and translation equivariance under wrap mode."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def images():
    sys.path.insert(0, str(ROOT))
    import bench

    return {"robust": bench.robust_image(4096), "gaussian": bench.gaussian_image(2048)}


def _gpu(image, kind, size, footprint=None, origin=None, mode="reflect", omit=True, parameter=0, q=50.0,
         ignore_inf=False, min_count=1):
    from ndfiltrs_gb300 import _core

    window = footprint.shape if footprint is not None else size
    with _core.Plan(image.shape, image.dtype, kind, window, footprint=footprint, origin=origin,
                    mode=[mode] * image.ndim, omit_nan=omit, parameter=parameter, percentile=q,
                    ignore_inf=ignore_inf, min_count=min_count) as plan:
        return plan.run_host(image), plan.algorithm


def _strip_check(oracle, image, result, kind, size, footprint=None, origin=None, mode="reflect", omit=True,
                 parameter=0, q=50.0, strips=3, rows=12, seed=0, ignore_inf=False, min_count=1, cval=0.0):
    """Compare `rows`-row strips (top, bottom, random interior) with the
    oracle run on crops of the rows those windows read, mapped through the
    image's vertical boundary mode (so every compared row sees exactly the
    samples of the full image)."""
    window = footprint.shape if footprint is not None else size
    kh = window[0]
    oy = 0 if origin is None else origin[0]
    anchor = kh // 2 + oy
    height = image.shape[0]
    rng = np.random.default_rng(seed)
    starts = [0, height - rows] + [int(v) for v in rng.integers(kh, height - rows - kh, size=strips)]
    for y0 in starts:
        sources = [oracle.map_index(y, height, mode) for y in range(y0 - anchor, y0 + rows + kh - 1 - anchor)]
        crop = np.stack([image[m] if m is not None else np.full(image.shape[1:], cval, image.dtype)
                         for m in sources])
        expected = oracle.window_filter(np.ascontiguousarray(crop), kind, window, footprint=footprint,
                                        origin=0 if origin is None else origin, mode=mode, omit_nan=omit,
                                        parameter=parameter, q=q, ignore_inf=ignore_inf, min_count=min_count,
                                        cval=cval)
        np.testing.assert_array_equal(bits(result[y0:y0 + rows]), bits(expected[anchor:anchor + rows]),
                                      err_msg=str((y0, mode)))


def test_config1_direct_3x3_2048(gpu, oracle, images) -> None:
    image = images["gaussian"]
    result, algorithm = _gpu(image, "median", (3, 3))
    _strip_check(oracle, image, result, "median", (3, 3))
    lo, _ = _gpu(image, "min", (3, 3))
    hi, _ = _gpu(image, "max", (3, 3))
    finite = np.isfinite(result)
    assert np.all(lo[finite] <= result[finite]) and np.all(result[finite] <= hi[finite])


@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
def test_config2_robust_4096_all_modes(gpu, oracle, images, mode) -> None:
    from ndfiltrs_gb300 import kernels

    image = images["robust"]
    ring = kernels.ring(4, 6, 2) != 0
    tophat = kernels.tophat(1, 2) != 0
    for kind, size, fp, omit, parameter, q in (("median_network", (5, 5), None, True, 0, 50.0),
                                               ("rank", (5, 5), None, False, 2, 50.0),
                                               ("percentile", (7, 7), None, True, 0, 84.0),
                                               ("median_network", None, ring, True, 0, 50.0),
                                               ("percentile", None, tophat, True, 0, 16.0)):
        result, _ = _gpu(image, kind, size, fp, (1, -1), mode, omit, parameter, q)
        _strip_check(oracle, image, result, kind, size, fp, (1, -1), mode, omit, parameter, q, strips=1, rows=6,
                     seed=hash(mode) % 1000)


def test_config2_properties(gpu, images) -> None:
    image = images["robust"]
    p16, _ = _gpu(image, "percentile", (7, 7), q=16.0)
    p50, _ = _gpu(image, "percentile", (7, 7), q=50.0)
    p84, _ = _gpu(image, "percentile", (7, 7), q=84.0)
    ok = np.isfinite(p16) & np.isfinite(p84)
    assert np.all(p16[ok] <= p50[ok]) and np.all(p50[ok] <= p84[ok])
    ranks = [_gpu(image, "rank", (5, 5), omit=False, parameter=k)[0] for k in (1, 2, 3)]
    ok = np.isfinite(ranks[0]) & np.isfinite(ranks[2])
    assert np.all(ranks[0][ok] <= ranks[1][ok]) and np.all(ranks[1][ok] <= ranks[2][ok])
    # Translation equivariance with wrap mode.
    shifted = np.ascontiguousarray(np.roll(image, (37, -91), axis=(0, 1)))
    a, _ = _gpu(image, "median_network", (5, 5), mode="wrap")
    b, _ = _gpu(shifted, "median_network", (5, 5), mode="wrap")
    np.testing.assert_array_equal(bits(np.roll(a, (37, -91), axis=(0, 1))), bits(b))


def test_config2_cube(gpu, oracle) -> None:
    sys.path.insert(0, str(ROOT))
    import bench

    cube = bench.cube_image()
    result, algorithm = _gpu(cube, "median_network", (3, 5, 5))
    # Leading slab (z edge) and an interior slab with its z halo.
    for z0 in (0, 30):
        lo = max(0, z0 - 1)
        crop = np.ascontiguousarray(cube[lo:z0 + 3])
        expected = oracle.window_filter(crop, "median_network", (3, 5, 5), mode="reflect", omit_nan=True)
        rows = slice(z0 - lo, z0 - lo + 2) if z0 else slice(0, 2)
        np.testing.assert_array_equal(bits(result[z0:z0 + 2]), bits(expected[rows]))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_config3_sky_8192_histogram(gpu, oracle, dtype) -> None:
    sys.path.insert(0, str(ROOT))
    import bench

    sky = bench.sky_image(8192, dtype=dtype)
    for size in ((65, 65), (129, 129)):
        result, algorithm = _gpu(sky, "median_histogram", size, mode="nearest")
        assert algorithm == "histogram"
        _strip_check(oracle, sky, result, "median", size, mode="nearest", strips=1, rows=4, seed=size[0])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_config4_precision_full_size(gpu, oracle, dtype) -> None:
    """nanstd on the full 4096^2 precision image: strips against the exact
    (double-double) moments oracle within 2 ulp (float32) / 1e-12 (float64)."""
    sys.path.insert(0, str(ROOT))
    import bench

    image = bench.precision_image(4096, dtype=dtype)
    for size in ((31, 31), (7, 51)):
        result, _ = _gpu(image, "std", size, parameter=1, ignore_inf=True, min_count=5)
        for y0 in (0, 2001):
            lo = max(0, y0 - size[0] // 2)
            crop = np.ascontiguousarray(image[lo:y0 + 8 + size[0] // 2])
            exact = oracle.exact_moments(crop, "std", size, mode="reflect", ddof=1, omit_nan=True,
                                         ignore_inf=True, min_count=5)[y0 - lo:y0 - lo + 8]
            got = result[y0:y0 + 8].astype(np.float64)
            assert np.array_equal(np.isnan(got), np.isnan(exact))
            ok = np.isfinite(exact) & (exact > 0)
            if dtype == np.float32:
                ulp = np.spacing(np.abs(exact[ok].astype(np.float32))).astype(np.float64)
                assert np.all(np.abs(got[ok] - exact[ok]) <= 2 * ulp)
            else:
                assert np.all(np.abs(got[ok] - exact[ok]) <= 1e-12 * np.abs(exact[ok]))
