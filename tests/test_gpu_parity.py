"""CUDA library vs the CPU oracle on seeded inputs.

Order statistics (median / sortnet / histogram, rank, min, max, percentile)
must be bit-identical. Mean/var/std are bit-identical on the FP64 path and
within the stated tolerance on the FP32-compensated path: 2 ulp of float32
output, and 1e-12 relative for float64 output (relative to the window's
deviation scale, see ``_moment_tolerance``).
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu

MODES = ("reflect", "constant", "nearest", "mirror", "wrap")
SELECTIONS = ("median", "median_network", "rank", "min", "max", "percentile")


def _special_values(shape, dtype, seed, fraction=0.12):
    """Values with ties, signed zeros, infinities and NaN payloads
    (tests/test_histogram_median.py:29-43 style)."""
    rng = np.random.default_rng(seed)
    values = (rng.integers(-6, 7, size=shape) / 4).astype(dtype)
    if values.size:
        values += rng.normal(size=shape).astype(dtype) * dtype(0.01)
    payload = np.array([0xFFC01234 if dtype == np.float32 else 0xFFF8000000001234],
                       dtype=np.uint32 if dtype == np.float32 else np.uint64).view(dtype)[0]
    special = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, np.finfo(dtype).max, payload], dtype=dtype)
    chosen = rng.random(shape) < fraction
    values[chosen] = rng.choice(special, size=int(chosen.sum()))
    return values


def _gpu(kind, array, size, footprint, origin, mode, cval, omit, ignore_inf, min_count, parameter=0, q=50.0,
         moments=None):
    from ndfiltrs_gb300 import _core

    if footprint is not None:
        size = list(np.asarray(footprint).shape)
    if kind == "percentile":
        return _core.robust_filter(array, size, footprint, origin, mode, cval, "percentile", q, omit,
                                   ignore_inf if omit else False, min_count if omit else 1,
                                   3.0, 3.0, 5, "median", "std")
    with _core.Plan(array.shape, array.dtype, kind, size, footprint=footprint, origin=origin,
                    mode=mode, cval=cval, omit_nan=omit, ignore_inf=ignore_inf,
                    min_count=min_count, parameter=parameter, moments=moments) as plan:
        return plan.run_host(np.ascontiguousarray(array))


def _oracle(oracle, kind, array, size, footprint, origin, mode, cval, omit, ignore_inf, min_count,
            parameter=0, q=50.0):
    return oracle.window_filter(array, kind, size, footprint=footprint, origin=origin, mode=mode,
                                cval=cval, omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count,
                                parameter=parameter, q=q)


def _assert_bits(actual, expected, context):
    np.testing.assert_array_equal(bits(actual), bits(expected), err_msg=str(context))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", MODES)
def test_selection_kinds_all_policies_2d(gpu, oracle, dtype, mode) -> None:
    values = _special_values((37, 45), dtype, seed=11)
    for size, origin in (((3, 3), (0, 0)), ((5, 4), (1, -2)), ((2, 7), (-1, 3)), ((1, 1), (0, 0))):
        volume = int(np.prod(size))
        for omit, ignore_inf, min_count in ((False, False, 1), (True, False, 1),
                                            (True, True, (volume + 1) // 2), (True, True, volume)):
            for kind in SELECTIONS:
                params = [0]
                if kind == "rank":
                    params = sorted({0, volume // 3, volume - 1})
                for parameter in params:
                    for q in ((16.0, 84.0, 100.0) if kind == "percentile" else (50.0,)):
                        args = (kind, values, size, None, origin, (mode, mode), 0.5, omit,
                                ignore_inf, min_count, parameter, q)
                        _assert_bits(_gpu(*args), _oracle(oracle, *args), args[:1] + args[2:])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_histogram_kinds_match_direct(gpu, oracle, dtype) -> None:
    values = _special_values((70, 66), dtype, seed=5)
    for size, origin, mode in (((3, 3), (0, 0), "reflect"), ((6, 5), (-3, 2), "wrap"),
                               ((2, 41), (0, -20), "mirror"), ((35, 3), (0, 0), "constant"),
                               ((33, 31), (0, 0), "nearest"), ((1, 9), (0, 4), "reflect")):
        volume = int(np.prod(size))
        for omit, ignore_inf, min_count in ((False, False, 1), (True, False, 1), (True, True, volume // 2 + 1)):
            for kind, parameter in (("median_histogram", 0), ("rank_histogram", 0),
                                    ("rank_histogram", volume // 3), ("rank_histogram", volume - 1)):
                args = (kind, values, size, None, origin, (mode, mode), -0.0, omit, ignore_inf,
                        min_count, parameter)
                expected = _oracle(oracle, kind.replace("_histogram", "") if kind != "median_histogram"
                                   else "median", *args[1:])
                _assert_bits(_gpu(*args), expected, (kind, size, origin, mode, omit, ignore_inf))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_every_network_width_and_radix(gpu, oracle, dtype) -> None:
    """Tap counts around each register-network width (8..128) and beyond it
    (the radix-select kernel), with footprints."""
    rng = np.random.default_rng(7)
    values = _special_values((29, 41), dtype, seed=3)
    for count in (1, 2, 5, 8, 9, 16, 17, 25, 32, 33, 49, 64, 65, 68, 100, 128, 129, 200, 300):
        side = int(np.ceil(np.sqrt(count))) + 1
        flat = np.zeros(side * side, dtype=bool)
        flat[rng.choice(side * side, size=count, replace=False)] = True
        footprint = flat.reshape(side, side)
        for omit, min_count in ((False, 1), (True, max(1, count // 3))):
            for kind in ("median", "rank", "percentile"):
                parameter = count // 2 if kind == "rank" else 0
                args = (kind, values, None, footprint, (0, 0), ("reflect", "wrap"), 1.5, omit, False,
                        min_count, parameter, 84.0)
                _assert_bits(_gpu(*args), _oracle(oracle, *args), (count, kind, omit))


@pytest.mark.parametrize("family,algorithm", [("ranked", "rank_network"), ("network", "tile_network")])
def test_ranked_and_plain_networks_every_width(gpu, oracle, family, algorithm) -> None:
    """Float32 windows of 33 to 128 taps on the ranked network kernel (16-bit
    rank codes, two windows per thread; 2-D windows) and, pinned, on the plain
    register network: rings, random footprints, boxes and a 3-D box, every selection
    kind, both NaN policies with ignore_inf and min_count, boundary modes with
    a non-zero cval, arrays of several 64-wide tiles with ragged edges; bit
    for bit against the oracle."""
    from ndfiltrs_gb300 import _core, kernels

    rng = np.random.default_rng(19)
    plane = _special_values((150, 171), np.float32, seed=21, fraction=0.05)
    cube = _special_values((5, 70, 97), np.float32, seed=22, fraction=0.05)
    windows = [(plane, kernels.ring(4, 6, 2) != 0, None), (plane, None, (7, 9)), (plane, None, (9, 9)),
               (plane, None, (11, 11)), (cube, None, (3, 5, 5))]
    for count in (33, 49, 75, 100, 128):
        flat = np.zeros(13 * 13, dtype=bool)
        flat[rng.choice(13 * 13, size=count, replace=False)] = True
        windows.append((plane, flat.reshape(13, 13), None))
    cases = [("median", 0, True, False, 1, ("reflect", "mirror")), ("median", 0, False, False, 1, ("nearest", "wrap")),
             ("median", 0, True, True, 20, ("constant", "reflect")), ("rank", 7, True, False, 1, ("wrap", "nearest")),
             ("percentile", 0, True, False, 1, ("mirror", "constant")), ("min", 0, False, False, 1, ("reflect",) * 2),
             ("max", 0, True, True, 1, ("nearest", "mirror"))]
    _core.pin_kernel(family)
    try:
        for values, footprint, size in windows:
            for kind, parameter, omit, ignore_inf, min_count, mode2 in cases:
                mode = mode2 if values.ndim == 2 else ("reflect",) + mode2
                origin = (0,) * values.ndim
                if kind != "percentile":
                    shape = size if footprint is None else footprint.shape
                    with _core.Plan(values.shape, np.float32, kind, shape, footprint=footprint, origin=origin,
                                    mode=mode, cval=-0.75, omit_nan=omit, ignore_inf=ignore_inf,
                                    min_count=min_count, parameter=parameter) as plan:
                        # 3-D windows keep the plain network (the ranked kernel
                        # would rank kd planes of support per output plane).
                        expected = algorithm if values.ndim == 2 else "tile_network"
                        assert plan.algorithm == expected, (plan.algorithm, kind, size)
                args = (kind, values, size, footprint, origin, mode, -0.75, omit, ignore_inf, min_count, parameter,
                        84.0)
                context = (family, kind, size, None if footprint is None else int(footprint.sum()), omit)
                _assert_bits(_gpu(*args), _oracle(oracle, *args), context)
    finally:
        _core.pin_kernel(None)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ranks_one_to_five(gpu, oracle, dtype) -> None:
    cases = [
        ((150,), (7,), (2,), ("mirror",)),
        ((1, 90), (4, 7), (1, 0), ("wrap", "nearest")),
        ((9, 40, 37), (3, 2, 5), (-1, 0, 2), ("mirror", "reflect", "constant")),
        ((6, 20, 21), (3, 5, 5), (0, 0, 0), ("reflect",) * 3),
        ((3, 4, 5, 6), (3, 1, 3, 2), (0, 0, 1, 0), ("reflect", "constant", "wrap", "nearest")),
        ((2, 2, 2, 2, 3), (3, 3, 3, 3, 5), (0,) * 5, ("reflect", "constant", "nearest", "mirror", "wrap")),
    ]
    for shape, size, origin, mode in cases:
        values = _special_values(shape, dtype, seed=len(shape))
        for kind in ("median", "median_network", "rank", "percentile", "max"):
            for omit in (False, True):
                args = (kind, values, size, None, origin, mode, -4.0, omit, False, 1,
                        int(np.prod(size)) // 4, 16.0)
                _assert_bits(_gpu(*args), _oracle(oracle, *args), (shape, kind, omit))


def _moment_tolerance(actual, expected, dtype, context):
    """FP32-compensated moments: <= 2 ulp (float32 output) or <= 1e-12
    relative (float64 output) where the result is a normal number."""
    np.testing.assert_array_equal(np.isnan(actual), np.isnan(expected), err_msg=str(context))
    finite = np.isfinite(expected) & (np.abs(expected) > np.finfo(dtype).tiny * 1e6)
    a = actual[finite].astype(np.float64)
    e = expected[finite].astype(np.float64)
    if dtype == np.float32:
        ulp = np.spacing(np.abs(expected[finite])).astype(np.float64)
        assert np.all(np.abs(a - e) <= 2 * ulp), context
    else:
        rel = np.abs(a - e) / np.abs(e)
        assert np.all(rel <= 1e-12), (context, float(rel.max(initial=0)))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("mode", MODES)
def test_moments_fp64_bit_exact_and_fp32c_tolerance(gpu, oracle, dtype, mode) -> None:
    rng = np.random.default_rng(4)
    base = (1e4 + rng.normal(size=(33, 47))).astype(dtype)
    base[rng.random(base.shape) < 0.05] = np.nan
    specials = _special_values((33, 47), dtype, seed=9)
    for values, tol_ok in ((base, True), (specials, False)):
        for size, footprint, origin in (((5, 5), None, (0, 0)), ((3, 7), None, (1, -2)),
                                        (None, np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]]), (0, 0))):
            for kind in ("mean", "var", "std"):
                for omit, ignore_inf, min_count, ddof in ((False, False, 1, 0), (True, True, 3, 1),
                                                          (True, False, 1, 1)):
                    args = (kind, values, size, footprint, origin, (mode, mode), 2.0, omit, ignore_inf,
                            min_count, ddof)
                    expected = _oracle(oracle, *args)
                    exact = _gpu(*args, moments="fp64")
                    _assert_bits(exact, expected, (kind, size, omit, "fp64"))
                    fast = _gpu(*args, moments="fp32c")
                    if tol_ok:
                        _moment_tolerance(fast, expected, dtype, (kind, size, omit, "fp32c"))
                    else:
                        np.testing.assert_array_equal(np.isnan(fast), np.isnan(expected))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_moments_generic_rank4(gpu, oracle, dtype) -> None:
    values = _special_values((3, 4, 5, 6), dtype, seed=21)
    for kind in ("mean", "var", "std"):
        for omit in (False, True):
            args = (kind, values, (3, 1, 3, 2), None, (0, 0, 1, 0),
                    ("reflect", "constant", "wrap", "nearest"), -1.0, omit, False, 1, 1)
            _assert_bits(_gpu(*args, moments="fp64"), _oracle(oracle, *args), (kind, omit))


def test_empty_and_degenerate_shapes(gpu, oracle) -> None:
    for shape in ((0, 3), (2, 0, 3), (2, 3, 0)):
        for kind in ("median", "mean", "rank"):
            out = _gpu(kind, np.empty(shape, np.float32), (3,) * len(shape), None, (0,) * len(shape),
                       ("wrap",) * len(shape), 0.0, False, False, 1)
            assert out.shape == shape and out.size == 0
    # Windows much larger than the array (multi-period boundary mapping).
    values = _special_values((3, 4), np.float64, seed=2)
    for mode in MODES:
        for kind in ("median", "percentile", "mean"):
            args = (kind, values, (9, 11), None, (0, 0), (mode, mode), 3.0, True, False, 1, 0, 84.0)
            expected = _oracle(oracle, *args)
            actual = _gpu(*args, moments="fp64") if kind == "mean" else _gpu(*args)
            _assert_bits(actual, expected, (mode, kind))


def test_large_window_medians(gpu, oracle) -> None:
    """A 65x65 window (histogram / radix paths) on a sky-like image crop."""
    rng = np.random.default_rng(3)
    y, x = np.mgrid[0:160, 0:170]
    sky = 500 + 0.01 * x - 0.005 * y
    image = (sky + rng.normal(size=sky.shape) * np.sqrt(sky)).astype(np.float32)
    image[:, 37] = np.nan
    for kind in ("median", "median_histogram"):
        for dtype in (np.float32, np.float64):
            args = (kind, image.astype(dtype), (65, 65), None, (0, 0), ("nearest", "nearest"), 0.0,
                    True, False, 1)
            _assert_bits(_gpu(*args), _oracle(oracle, "median", *args[1:]), (kind, dtype))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("box", [3, 5, 7])
def test_box_pair_kernel(gpu, oracle, dtype, box) -> None:
    """3x3 / 5x5 / 7x7 windows (the vertical-pair box kernel) over partial
    tiles, every mode, shifted origins, all policies and selection kinds."""
    from ndfiltrs_gb300 import _core

    values = _special_values((45, 70), dtype, seed=box)
    volume = box * box
    for mode in MODES:
        for origin in ((0, 0), (box // 2, -(box // 2)), (-1, 1)):
            for omit, ignore_inf, min_count in ((False, False, 1), (True, False, 1), (True, True, volume // 2)):
                for kind, parameter, q in (("median", 0, 50.0), ("median_network", 0, 50.0),
                                           ("rank", 2, 50.0), ("rank", volume - 1, 50.0),
                                           ("min", 0, 50.0), ("max", 0, 50.0), ("percentile", 0, 84.0)):
                    args = (kind, values, (box, box), None, origin, (mode, mode), 0.25, omit, ignore_inf,
                            min_count, parameter, q)
                    _assert_bits(_gpu(*args), _oracle(oracle, *args), (box, mode, origin, omit, kind))
    plan = _core.Plan(values.shape, dtype, "median", (box, box), omit_nan=True)
    if dtype == np.float32 or box < 7:
        assert plan.algorithm == "tile_box"
    plan.close()


def test_float32_midpoint_fast_path_matches_float64_rule(gpu, oracle) -> None:
    """Even-count medians over value pairs that straddle every branch of the
    float32 midpoint fast path (exponent gaps around 28, tiny and huge
    magnitudes, signed zeros, opposite signs) stay bit-identical."""
    rng = np.random.default_rng(99)
    specials = np.array([0.0, -0.0, 1.0, -1.0, 3.4e38, -3.4e38, 1e-30, -1e-30, 1e-38, 2.0 ** -97,
                         2.0 ** -98, 2.0 ** 126, 2.0 ** 127, 1.0 + 2.0 ** -23, 2.0 ** 28, 2.0 ** 29,
                         1.5e-45, np.inf, -np.inf], dtype=np.float32)
    mags = (2.0 ** rng.integers(-140, 128, size=4000)).astype(np.float32)
    values = np.concatenate([specials, mags * rng.choice([-1, 1], size=mags.size),
                             rng.normal(size=4000).astype(np.float32) * 1000])
    rng.shuffle(values)
    pairs = values[: (values.size // 2) * 2].reshape(-1, 2)
    # Each 2-sample window (size 2, wrap over a 2-long axis) is one midpoint.
    array = np.ascontiguousarray(pairs, dtype=np.float32)
    for kind in ("median", "median_network"):
        args = (kind, array, (1, 2), None, (0, 0), ("wrap", "wrap"), 0.0, True, False, 1)
        _assert_bits(_gpu(*args), _oracle(oracle, "median", *args[1:]), kind)
    # The same pairs inside 3x3 windows with one NaN (8 retained samples).
    grid = np.resize(values, (40, 60)).astype(np.float32)
    grid[::3, ::3] = np.nan
    for kind in ("median", "median_network"):
        args = (kind, grid, (3, 3), None, (0, 0), ("reflect", "reflect"), 0.0, True, False, 1)
        _assert_bits(_gpu(*args), _oracle(oracle, "median", *args[1:]), kind)


def _disk(radius):
    y, x = np.mgrid[-radius:radius + 1, -radius:radius + 1]
    return (x * x + y * y) <= radius * radius


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_footprint_histogram(gpu, oracle, dtype) -> None:
    """Footprints beyond the register networks (> 128 taps) slide the rank
    histogram by the ends of the footprint's runs: disks, rings, masks with
    holes and empty border rows/columns, over multi-tile images with partial
    tiles, every mode and shifted origins."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(21)
    holes = _disk(8)
    holes[rng.random(holes.shape) < 0.3] = False
    ring = _disk(9) & ~np.pad(_disk(6), 3)
    bordered = np.zeros((15, 17), dtype=bool)
    bordered[2:13, 1:15] = _disk(7)[2:13, 0:14] | (rng.random((11, 14)) < 0.2)
    footprints = {"disk7": _disk(7), "ring9": ring, "holes": holes, "bordered": bordered}
    values = _special_values((83, 150), dtype, seed=5, fraction=0.05)
    for name, footprint in footprints.items():
        assert footprint.sum() > 128, name
        with _core.Plan(values.shape, dtype, "median", footprint.shape, footprint=footprint,
                        omit_nan=True) as plan:
            assert plan.algorithm == "histogram", name
        for mode in MODES:
            origin = (0, 0) if mode in ("reflect", "wrap") else (1, -2)
            for omit, ignore_inf, min_count in ((False, False, 1), (True, True, 40)):
                for kind, parameter, q in (("median", 0, 50.0), ("rank", 7, 50.0), ("min", 0, 50.0),
                                           ("max", 0, 50.0), ("percentile", 0, 84.0)):
                    args = (kind, values, None, footprint, origin, (mode, mode), -0.75, omit, ignore_inf,
                            min_count, parameter, q)
                    _assert_bits(_gpu(*args), _oracle(oracle, *args), (name, mode, omit, kind))


def test_footprint_histogram_1d_and_small_arrays(gpu, oracle) -> None:
    rng = np.random.default_rng(8)
    mask = rng.random(301) < 0.6
    mask[0] = mask[-1] = True
    line = _special_values((1000,), np.float32, seed=1, fraction=0.05)
    for mode in MODES:
        for kind in ("median", "percentile", "rank"):
            args = (kind, line, None, mask, (3,), (mode,), 2.0, True, False, 1, 11, 16.0)
            _assert_bits(_gpu(*args), _oracle(oracle, *args), (mode, kind))
    # An image smaller than the footprint (every sample is boundary-mapped).
    small = _special_values((6, 9), np.float64, seed=4, fraction=0.1)
    for mode in MODES:
        args = ("median", small, None, _disk(7), (0, 0), (mode, mode), 1.0, True, False, 1)
        _assert_bits(_gpu(*args), _oracle(oracle, *args), mode)


def test_float32_percentile_fast_path_matches_float64_rule(gpu, oracle) -> None:
    """Percentile interpolation of float32 samples (three float64 operations
    and an integer float64 -> float32 rounding in the common case) stays
    bit-identical to the reference's float64 rule for many q, over values of
    every magnitude, subnormals, signed zeros and mixed signs, in the box,
    register-network and histogram kernels."""
    rng = np.random.default_rng(1234)
    mags = (2.0 ** rng.uniform(-149, 127, size=(61, 67))).astype(np.float32)
    wide = mags * rng.choice(np.array([-1, 1], dtype=np.float32), size=mags.shape)
    near = (1000 + rng.normal(size=(61, 67)) * 1e-3).astype(np.float32)
    for values in (wide, near, _special_values((61, 67), np.float32, seed=31)):
        for q in (0.0, 0.1, 12.5, 33.3, 50.0, 66.7, 84.0, 99.9, 100.0):
            for size, footprint in (((5, 5), None), ((7, 7), None), (None, _disk(3)),
                                    ((15, 15), None), (None, _disk(7))):
                args = ("percentile", values, size, footprint, (0, 0), ("reflect", "mirror"), 0.0, True,
                        False, 1, 0, q)
                _assert_bits(_gpu(*args), _oracle(oracle, *args), (q, size))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sliding_moments_against_exact_oracle(gpu, oracle, dtype) -> None:
    """FP32C boxes run the sliding exact-sum kernel: within 2 ulp (float32) /
    1e-12 relative (float64) of the exact (double-double) window moments,
    under every mode, policy and ddof, with NaN / infinity classification
    equal to the reference's; tiles whose value range is too wide for the
    integer widths take the per-window paths (checked the same way)."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(31)
    smooth = (1e4 + rng.normal(size=(90, 110))).astype(dtype)
    smooth[rng.random(smooth.shape) < 0.03] = np.nan
    smooth[rng.random(smooth.shape) < 0.01] = np.inf
    steps = (np.where(np.arange(110)[None, :] < 55, 1e3, 6e4) + rng.normal(size=(90, 110)) * 10).astype(dtype)
    wide = (rng.normal(size=(90, 110)) * 10.0 ** rng.integers(-30, 30, size=(90, 110))).astype(dtype)
    line = (5 + rng.normal(size=(1, 700))).astype(dtype)
    for values, size in ((smooth, (7, 9)), (steps, (5, 13)), (wide, (3, 4)), (line, (1, 31))):
        for mode in MODES:
            for kind in ("mean", "var", "std"):
                for omit, ignore_inf, min_count, ddof in ((True, True, 5, 1), (False, False, 1, 0),
                                                          (True, False, 1, 2)):
                    with _core.Plan(values.shape, dtype, kind, size, mode=[mode] * 2, cval=1.5, omit_nan=omit,
                                    ignore_inf=ignore_inf, min_count=min_count,
                                    parameter=ddof if kind != "mean" else 0) as plan:
                        assert plan.algorithm == "moments_slide"
                        actual = plan.run_host(values)
                    exact = oracle.exact_moments(values, kind, size, mode=mode, cval=1.5, omit_nan=omit,
                                                 ignore_inf=ignore_inf, min_count=min_count,
                                                 ddof=ddof if kind != "mean" else 0)
                    # Windows whose value range forces the reference's float64
                    # arithmetic (the "wide" image) must equal it bit for bit
                    # instead: under heavy cancellation that arithmetic is
                    # itself not within the tolerance of the exact moments.
                    reference = oracle.window_filter(values, kind, size, mode=mode, cval=1.5, omit_nan=omit,
                                                     ignore_inf=ignore_inf, min_count=min_count,
                                                     parameter=ddof if kind != "mean" else 0)
                    context = (values.shape, size, mode, kind, omit, ddof)
                    np.testing.assert_array_equal(np.isnan(actual), np.isnan(exact), err_msg=str(context))
                    ok = np.isfinite(exact) & (np.abs(exact) > np.finfo(dtype).tiny * 1e6)
                    np.testing.assert_array_equal(actual[np.isinf(exact)], exact[np.isinf(exact)].astype(dtype))
                    a, e = actual[ok].astype(np.float64), exact[ok]
                    if dtype == np.float32:
                        ulp = np.spacing(np.abs(e.astype(np.float32))).astype(np.float64)
                        close = np.abs(a - e) <= 2 * ulp
                    else:
                        close = np.abs(a - e) <= 1e-12 * np.abs(e)
                    same_as_reference = bits(actual[ok]) == bits(reference[ok])
                    assert np.all(close | same_as_reference), context
                    if values is not wide:
                        assert np.all(close), context


def _slide_path_images(rng, dtype):
    """Images that steer the sliding moments kernel's tiles into each of its
    arithmetic paths (name, array)."""
    shape = (150, 170)
    base = 1e4 + rng.normal(size=shape)
    images = [("finite", base)]
    for name, value in (("nan_only", np.nan), ("pinf_only", np.inf), ("ninf_only", -np.inf)):
        image = base.copy()
        image[rng.random(shape) < 0.02] = value
        image[40:47, 60:70] = value  # windows with many of them
        images.append((name, image))
    mixed = base.copy()
    mixed[rng.random(shape) < 0.02] = np.nan
    mixed[rng.random(shape) < 0.01] = np.inf
    mixed[rng.random(shape) < 0.01] = -np.inf
    images.append(("mixed", mixed))
    # Multiples of 1/8 up to 2^24: deviations of about 28 bits, whose window
    # sums of squares need 128 bits.
    images.append(("eighths", np.round(rng.uniform(-2.0**24, 2.0**24, size=shape) * 8) / 8))
    # A column of tiny values: deviations beyond 30 (float32) bits.
    tiny = base.copy()
    tiny[:, 33] *= 1e-7
    tiny[rng.random(shape) < 0.01] = np.nan
    images.append(("tiny_column", tiny))
    # Small integers: narrow sums for float64 too.
    integers = np.floor(rng.normal(100.0, 20.0, size=shape))
    integers[rng.random(shape) < 0.02] = np.nan
    images.append(("integers", integers))
    return [(name, image.astype(dtype)) for name, image in images]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sliding_moments_every_path_is_exact(gpu, oracle, dtype) -> None:
    """The sliding moments kernel keeps 64- or 128-bit column sums, packs the
    count of a single non-finite class above the sum of deviations or keeps
    every class's counts, and holds deviations in place of the samples or
    recomputes them; every combination (steered by the images' value
    ranges and non-finite classes) stays within 1 ulp (float32) / 1e-15
    relative (float64) of the exact window moments, with the reference's
    NaN / infinity classification, under both NaN policies, both infinity
    policies, ddof, min_count and boundary modes, on tiles cut by the array
    edges."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(23)
    for name, values in _slide_path_images(rng, dtype):
        for size, mode in (((7, 9), "reflect"), ((31, 31), "nearest"), ((3, 45), "wrap"), ((33, 2), "constant")):
            for kind in ("mean", "var", "std"):
                for omit, ignore_inf, min_count, ddof in ((True, True, 5, 1), (False, False, 1, 0),
                                                          (True, False, 1, 2)):
                    parameter = ddof if kind != "mean" else 0
                    with _core.Plan(values.shape, dtype, kind, size, mode=[mode] * 2, cval=2.5, omit_nan=omit,
                                    ignore_inf=ignore_inf, min_count=min_count, parameter=parameter) as plan:
                        assert plan.algorithm == "moments_slide"
                        actual = plan.run_host(values)
                    exact = oracle.exact_moments(values, kind, size, mode=mode, cval=2.5, omit_nan=omit,
                                                 ignore_inf=ignore_inf, min_count=min_count, ddof=parameter)
                    context = (name, size, mode, kind, omit, ignore_inf, ddof)
                    np.testing.assert_array_equal(np.isnan(actual), np.isnan(exact), err_msg=str(context))
                    np.testing.assert_array_equal(actual[np.isinf(exact)], exact[np.isinf(exact)].astype(dtype),
                                                  err_msg=str(context))
                    finite = np.isfinite(exact) & (np.abs(exact) > np.finfo(dtype).tiny * 1e6)
                    a, e = actual[finite].astype(np.float64), exact[finite]
                    if dtype == np.float32:
                        ulp = np.spacing(np.abs(e.astype(np.float32))).astype(np.float64)
                        worst = float((np.abs(a - e) / ulp).max(initial=0))
                        assert worst <= 1, (context, worst)
                    else:
                        worst = float((np.abs(a - e) / np.abs(e)).max(initial=0))
                        assert worst <= 1e-15, (context, worst)


@pytest.mark.parametrize("family,algorithm", [("passes", "extrema_passes"), ("extrema", "extrema_tile")])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_separable_extrema(gpu, oracle, dtype, family, algorithm) -> None:
    """Rectangular minima / maxima run the separable (van Herk / Gil-Werman)
    kernels, the two column passes and the one-tile form: bit-identical to
    direct selection under every mode, origin and policy, with signed zeros,
    infinities, NaNs and NaN / infinite cval, on arrays that are not whole
    numbers of strips and blocks."""
    from ndfiltrs_gb300 import _core

    values = _special_values((97, 130), dtype, seed=13, fraction=0.06)
    tall = _special_values((301, 45), dtype, seed=15, fraction=0.02)
    line = _special_values((900,), dtype, seed=14, fraction=0.06)
    _core.pin_kernel(family)
    try:
        for array, size, origin in ((values, (9, 9), (1, -2)), (values, (33, 17), (-5, 3)),
                                    (values, (65, 65), (0, 0)), (values, (1, 31), (0, 7)),
                                    (tall, (129, 3), (60, -1)), (values, (3, 3), (0, 1)),
                                    (line, (41,), (-10,))):
            for mode in MODES:
                for kind in ("min", "max"):
                    for omit, ignore_inf, min_count, cval in ((False, False, 1, -0.5), (True, False, 1, np.nan),
                                                              (True, True, 9, np.inf), (False, False, 1, np.nan)):
                        args = (kind, array, size, None, origin, (mode,) * array.ndim, cval, omit, ignore_inf,
                                min_count)
                        with _core.Plan(array.shape, dtype, kind, size, origin=origin,
                                        mode=[mode] * array.ndim, cval=cval, omit_nan=omit,
                                        ignore_inf=ignore_inf, min_count=min_count) as plan:
                            assert plan.algorithm == algorithm
                            actual = plan.run_host(array)
                        _assert_bits(actual, _oracle(oracle, *args), (size, mode, kind, omit, ignore_inf, cval))
    finally:
        _core.pin_kernel(None)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_histogram_3d_windows(gpu, oracle, dtype) -> None:
    """3-D windows slide the rank histogram over supports of kd planes: boxes
    (walked through their run lists, as the reference's N-D histogram walks
    any rank, src/histogram.rs:494-566) and 3-D footprints (with the kernel
    family pinned), every boundary mode on every axis, shifted origins, both
    NaN policies, every order statistic; against the oracle bit for bit."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(33)
    values = _special_values((11, 45, 38), dtype, seed=9, fraction=0.08)
    footprint = rng.random((3, 7, 9)) < 0.7
    footprint[1, 3, 4] = True
    boxes = (((3, 5, 4), (0, 1, -1)), ((5, 9, 9), (-2, 0, 4)), ((4, 1, 6), (1, 0, 0)), ((2, 3, 1), (0, 1, 0)))
    for size, origin in boxes:
        with _core.Plan(values.shape, dtype, "median_histogram", size, origin=origin, omit_nan=True) as plan:
            assert plan.algorithm == "histogram", size
        for mode in MODES:
            modes = (mode, MODES[(MODES.index(mode) + 1) % 5], MODES[(MODES.index(mode) + 3) % 5])
            volume = int(np.prod(size))
            for omit, ignore_inf, min_count in ((False, False, 1), (True, True, max(1, volume // 3))):
                for kind, parameter in (("median_histogram", 0), ("rank_histogram", volume // 4)):
                    args = (kind, values, size, None, origin, modes, -1.25, omit, ignore_inf, min_count,
                            parameter)
                    base = "median" if kind == "median_histogram" else "rank"
                    _assert_bits(_gpu(*args), _oracle(oracle, base, *args[1:]), (size, modes, omit, kind))
    _core.pin_kernel("histogram")
    try:
        with _core.Plan(values.shape, dtype, "median", footprint.shape, footprint=footprint,
                        omit_nan=True) as plan:
            assert plan.algorithm == "histogram"
        for mode in MODES:
            for omit, ignore_inf, min_count in ((False, False, 1), (True, False, 9)):
                for kind, parameter, q in (("median", 0, 50.0), ("rank", 5, 50.0), ("min", 0, 50.0),
                                           ("max", 0, 50.0), ("percentile", 0, 16.0)):
                    args = (kind, values, None, footprint, (1, -2, 3), (mode,) * 3, 0.5, omit, ignore_inf,
                            min_count, parameter, q)
                    _assert_bits(_gpu(*args), _oracle(oracle, *args), ("footprint", mode, omit, kind))
    finally:
        _core.pin_kernel(None)


def test_histogram_3d_large_window(gpu, oracle) -> None:
    """A (9, 33, 33) window (9,801 taps) on a 12 x 100 x 90 cube: the sliding
    histogram against the oracle's direct selection, nearest and reflect."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(4)
    cube = (500 + rng.normal(size=(12, 100, 90)) * 20).astype(np.float32)
    cube[rng.random(cube.shape) < 0.01] = np.nan
    cube[:, :, 31] = np.nan
    size = (9, 33, 33)
    with _core.Plan(cube.shape, np.float32, "median_histogram", size, omit_nan=True) as plan:
        assert plan.algorithm == "histogram"
    for mode in ("nearest", "reflect"):
        for kind, parameter in (("median_histogram", 0), ("rank_histogram", 1234)):
            args = (kind, cube, size, None, (0, 0, 0), (mode,) * 3, 0.0, True, False, 1, parameter)
            base = "median" if kind == "median_histogram" else "rank"
            _assert_bits(_gpu(*args), _oracle(oracle, base, *args[1:]), (mode, kind))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fp32c_moments_are_exact_sums_rounded(gpu, oracle, dtype) -> None:
    """The default moments path sums exactly (fixed-point window sums), so on
    zero-centred data, where a compensated floating-point sum cancels, its
    results stay within 1 ulp (float32) / 1e-15 relative (float64) of the
    exact window moments, for boxes (sliding kernel) and footprints (tile
    kernel), every kind, with NaN / infinity handling and ddof."""
    from ndfiltrs_gb300 import kernels

    rng = np.random.default_rng(17)
    values = rng.normal(size=(61, 83)).astype(dtype)
    values[rng.random(values.shape) < 0.03] = np.nan
    values[rng.random(values.shape) < 0.01] = np.inf
    values[:, 7] *= dtype(1e-6)  # a column of tiny values widens the tiles' bit span
    ring = kernels.ring(2, 4, 2) != 0
    for size, footprint in (((9, 9), None), ((1, 31), None), (None, ring), (None, kernels.tophat(3, 2) != 0)):
        for kind in ("mean", "var", "std"):
            for ignore_inf, min_count, ddof in ((True, 1, 0), (True, 5, 1), (False, 1, 1)):
                args = (kind, values, size, footprint, (0, 0), ("reflect", "wrap"), 0.0, True, ignore_inf,
                        min_count, ddof)
                exact = oracle.exact_moments(values, kind, size, footprint=footprint, mode=("reflect", "wrap"),
                                             omit_nan=True, ignore_inf=ignore_inf, min_count=min_count, ddof=ddof)
                fast = _gpu(*args, moments="fp32c")
                context = (kind, size, None if footprint is None else int(footprint.sum()), ignore_inf, ddof)
                np.testing.assert_array_equal(np.isnan(fast), np.isnan(exact), err_msg=str(context))
                finite = np.isfinite(exact) & (np.abs(exact) > np.finfo(dtype).tiny * 1e6)
                np.testing.assert_array_equal(fast[np.isinf(exact)], exact[np.isinf(exact)].astype(dtype))
                a = fast[finite].astype(np.float64)
                e = exact[finite]
                if dtype == np.float32:
                    ulp = np.spacing(np.abs(e.astype(np.float32))).astype(np.float64)
                    assert np.all(np.abs(a - e) <= ulp), (context, float((np.abs(a - e) / ulp).max(initial=0)))
                else:
                    rel = np.abs(a - e) / np.abs(e)
                    assert np.all(rel <= 1e-15), (context, float(rel.max(initial=0)))
