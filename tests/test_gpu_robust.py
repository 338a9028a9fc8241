"""The robust family on the GPU: MAD, sigma clipping, mode, biweight.

Two kinds of checks:
* parity: every kind, both dtypes, all five modes, origins, footprints and
  policies, with NaN payloads, infinities, signed zeros, subnormals and
  magnitudes near the overflow threshold in the windows, bit for bit against
  the oracle's restatement of RobustReduction::finish (src/robust.rs:244-299,
  src/location.rs), including windows above 256 samples (the scratch-backed
  kernel);
* behaviour: the literal expectations of the reference's own Python tests
  (tests/test_robust.py, tests/test_location_filters.py of ysBach/ndfiltrs
  v0.2.0) through the public functions.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu

MODES = ("reflect", "constant", "nearest", "mirror", "wrap")
DTYPES = (np.float32, np.float64)

KIND_OPTIONS = {
    "mad": [dict(parameter=1.0), dict(parameter=2.5)],
    "mode": [dict(estimator="sex", pearson=2.5), dict(estimator="mmm", pearson=3.0),
             dict(estimator="iraf", pearson=3.0)],
    "biweight_location": [dict(parameter=6.0), dict(parameter=1.5)],
    "biweight_scale": [dict(parameter=9.0), dict(parameter=3.0, modify_sample_size=True)],
    "sigma_mean": [dict(sigma_lower=1.0, sigma_upper=1.0, maxiters=None),
                   dict(sigma_lower=2.0, sigma_upper=0.5, maxiters=2, center="mean", spread="mad")],
    "sigma_median": [dict(sigma_lower=1.5, sigma_upper=1.5, maxiters=5, spread="mad"),
                     dict(sigma_lower=0.0, sigma_upper=3.0, maxiters=0, center="mean")],
    "sigma_mode": [dict(sigma_lower=3.0, sigma_upper=3.0, maxiters=None, estimator="sex", pearson=2.5),
                   dict(sigma_lower=1.0, sigma_upper=2.0, maxiters=1, estimator="iraf", pearson=3.0)],
}


def _values(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    values = (100 + rng.normal(size=shape) * 10).astype(dtype)
    values[rng.random(shape) < 0.15] = dtype(100)  # ties: zero MADs and spreads
    info = np.finfo(dtype)
    special = np.array([np.nan, np.inf, -np.inf, -0.0, 0.0, info.smallest_subnormal, info.max,
                        -info.max, 1e-3], dtype=dtype)
    chosen = rng.random(shape) < 0.08
    values[chosen] = rng.choice(special, size=int(chosen.sum()))
    return values


def _gpu(array, kind, size, footprint, origin, mode, cval, omit, ignore_inf, min_count, options):
    from ndfiltrs_gb300 import _core

    clip = kind.startswith("sigma")
    opts = dict(options)
    args = dict(parameter=opts.pop("parameter", 0.0), sigma_lower=opts.pop("sigma_lower", 3.0),
                sigma_upper=opts.pop("sigma_upper", 3.0), maxiters=opts.pop("maxiters", 5),
                center=opts.pop("center", "median"), spread=opts.pop("spread", "std"),
                estimator=opts.pop("estimator", "sex"),
                modify_sample_size=opts.pop("modify_sample_size", False), pearson=opts.pop("pearson", 2.5))
    with _core.Plan(array.shape, array.dtype, kind, footprint.shape if footprint is not None else size,
                    footprint=footprint, origin=origin, mode=[mode] * array.ndim, cval=cval,
                    omit_nan=True if clip else omit, ignore_inf=True if clip else ignore_inf,
                    min_count=min_count, robust=args) as plan:
        assert plan.algorithm == "robust"
        return plan.run_host(np.ascontiguousarray(array))


def _oracle(oracle, array, kind, size, footprint, origin, mode, cval, omit, ignore_inf, min_count, options):
    return oracle.robust_filter(array, kind, size, footprint=footprint, origin=origin, mode=mode, cval=cval,
                                omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count, **options)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("kind", sorted(KIND_OPTIONS))
def test_robust_matches_oracle(gpu, oracle, kind, dtype) -> None:
    radius2 = np.add.outer(np.arange(-3, 4) ** 2, np.arange(-3, 4) ** 2)
    ring = (radius2 <= 9) & (radius2 > 2)
    # Windows of 25, 28, 9, 18 (register sort of 32), 49 and 64 (two
    # register-sorted runs merged) and 121 samples (insertion sort).
    cases = [((23, 31), (5, 5), None, (1, -2)), ((19, 26), None, ring, (0, 1)),
             ((40,), (9,), None, (3,)), ((5, 7, 6), (3, 2, 3), None, (0, 0, -1)),
             ((21, 19), (7, 7), None, (-1, 2)), ((18, 20), (8, 8), None, (0, -3)),
             ((17, 16), (11, 11), None, (0, 0))]
    clip = kind.startswith("sigma")
    for shape, size, footprint, origin in cases:
        values = _values(shape, dtype, seed=len(shape) * 13 + (size or (0,))[0])
        volume = int(np.count_nonzero(footprint)) if footprint is not None else int(np.prod(size))
        policies = [(False, False, 1), (True, False, 1), (True, True, max(2, volume // 3))]
        if clip:
            policies = [(True, True, 1), (True, True, max(2, volume // 3))]
        for options in KIND_OPTIONS[kind]:
            for mode in MODES:
                for omit, ignore_inf, min_count in policies:
                    for cval in (1.25, np.nan):
                        args = (values, kind, size, footprint, origin, mode, cval, omit, ignore_inf, min_count,
                                options)
                        actual = _gpu(*args)
                        expected = _oracle(oracle, *args)
                        np.testing.assert_array_equal(bits(actual), bits(expected),
                                                      err_msg=str((shape, mode, omit, min_count, cval, options)))


@pytest.mark.parametrize("dtype", DTYPES)
def test_robust_wide_windows_use_scratch(gpu, oracle, dtype) -> None:
    """17 x 17 = 289 samples per window: the scratch-backed kernel."""
    values = _values((40, 45), dtype, seed=21)
    for kind in ("mad", "biweight_scale", "sigma_median", "mode"):
        options = KIND_OPTIONS[kind][0]
        for mode in ("reflect", "constant"):
            args = (values, kind, (17, 17), None, (0, 0), mode, 3.0, True, False, 1, options)
            np.testing.assert_array_equal(bits(_gpu(*args)), bits(_oracle(oracle, *args)), err_msg=kind)


# ---------------------------------------------------------------------------
# Literal expectations of the reference's Python tests.

@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("mode", MODES)
def test_mad_matches_two_medians(gpu, dtype, mode) -> None:
    # tests/test_robust.py:43-56
    from scipy import ndimage

    nf = gpu
    array = np.array([[3, -4, 8], [1, 12, -2]], dtype=dtype)
    expected = ndimage.generic_filter(array, lambda v: 2 * np.median(np.abs(v - np.median(v))), size=(3, 5),
                                      mode=mode, cval=1.25)
    np.testing.assert_array_equal(nf.mad_filter(array, (3, 5), mode=mode, cval=1.25, scale=2), expected)


@pytest.mark.parametrize("dtype", DTYPES)
def test_mad_extremes_subnormals_and_policies(gpu, dtype) -> None:
    # tests/test_robust.py:59-68, 93-130, 155-199
    nf = gpu
    values = np.array([np.nan, 1, 3, 9, 11], dtype=dtype)
    np.testing.assert_array_equal(nf.nanmad_filter(values, 5, mode="wrap"), 4)
    np.testing.assert_array_equal(nf.nanmad_filter(values, 5, scale=2, mode="wrap"), 8)
    assert np.isnan(nf.nanmad_filter(values, 5, mode="wrap", min_count=5)).all()
    maximum = np.finfo(dtype).max
    np.testing.assert_array_equal(nf.mad_filter(np.array([-maximum, 0, maximum], dtype), mode="wrap"), maximum)
    np.testing.assert_array_equal(nf.mad_filter(np.array([-maximum, 0, maximum], dtype), mode="wrap", scale=0.5),
                                  maximum / 2)
    np.testing.assert_array_equal(nf.mad_filter(np.array([-maximum, -maximum, maximum], dtype), mode="wrap"), 0)
    smallest = np.nextafter(dtype(0), dtype(1))
    np.testing.assert_array_equal(nf.mad_filter(np.array([-smallest, 0, smallest], dtype), mode="wrap"), smallest)
    np.testing.assert_array_equal(nf.nanmad_filter(np.array([1, 3, np.inf], dtype), mode="wrap", ignore_inf=True), 1)
    assert np.isnan(nf.mad_filter(np.full(3, np.inf, dtype=dtype))).all()
    unsigned = np.uint32 if dtype is np.float32 else np.uint64
    canonical = 0x7FC00000 if dtype is np.float32 else 0x7FF8000000000000
    for result in (nf.mad_filter(np.array([1, np.nan, 3], dtype)), nf.nanmad_filter(np.full(3, np.nan, dtype)),
                   nf.sigma_clipped_filter(np.full(3, np.nan, dtype)),
                   nf.mad_filter(np.array([-np.inf, 0, np.inf], dtype), scale=0, mode="wrap")):
        np.testing.assert_array_equal(result.view(unsigned), canonical)


def test_mixed_modes_and_subnormal_clipping(gpu) -> None:
    # tests/test_robust.py:93-112, 141-152
    nf = gpu
    values = np.array([[[1.0, 2.0, 3.0]], [[10.0, 20.0, 30.0]]])
    np.testing.assert_array_equal(nf.mad_filter(values, (3, 1, 1), mode=("constant", "nearest", "wrap"), cval=5),
                                  [[[4, 3, 2]], [[4, 3, 2]]])
    tiny = np.nextafter(0.0, 1.0)
    np.testing.assert_array_equal(nf.nanmad_filter(np.array([0.0, tiny, np.nan]), scale=2, mode="wrap"), tiny)
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(np.array([0.0, tiny, tiny]), sigma=3, spread="std", center="median", min_count=3,
                                mode="wrap"), tiny)


@pytest.mark.parametrize("dtype", DTYPES)
def test_sigma_clipping_behaviour(gpu, dtype) -> None:
    # tests/test_robust.py:202-300
    nf = gpu
    values = np.array([0, 0, 0, 0, 1, 10, 100], dtype=dtype)
    for passes, expected in [(0, 111 / 7), (1, 11 / 6), (2, 0.2), (3, 0), (10, 0), (None, 0)]:
        actual = nf.sigma_clipped_filter(values, 7, sigma=1, maxiters=passes, mode="wrap")
        np.testing.assert_allclose(actual, dtype(expected), rtol=np.finfo(dtype).eps, atol=0)
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(np.array([1, 1, 1, 1, 100], dtype), 5, spread="mad", mode="wrap"), 1)
    values = np.array([-10, -1, -1, 0, 1, 1.4, 10], dtype=dtype)
    np.testing.assert_allclose(nf.sigma_clipped_filter(values, 7, spread="mad", sigma=1, maxiters=1, mode="wrap"),
                               dtype(np.mean(values[1:6].astype(np.float64))), rtol=np.finfo(dtype).eps, atol=0)
    values = np.array([-100, 0, 0, 0, 10], dtype=dtype)
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(values, 5, sigma_lower=10, sigma_upper=0.1, maxiters=1, mode="wrap"), -25)
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(values, 5, sigma_lower=0.1, sigma_upper=10, maxiters=1, mode="wrap"), 2.5)
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(np.array([-1, np.nan, 1], dtype), sigma=1, center="mean", min_count=2, mode="wrap"),
        0)
    np.testing.assert_array_equal(nf.sigma_clipped_filter(np.array([1, 1, 2], dtype), sigma=0, mode="wrap"), 1)
    values = np.array([1, 3, np.nan, np.inf, -np.inf], dtype=dtype)
    np.testing.assert_array_equal(nf.sigma_clipped_filter(values, 5, mode="wrap"), 2)
    assert np.isnan(nf.sigma_clipped_filter(values, 5, mode="wrap", min_count=3)).all()
    maximum = np.finfo(dtype).max
    np.testing.assert_array_equal(
        nf.sigma_clipped_filter(np.array([-maximum, np.nan, maximum], dtype), sigma=1, mode="wrap", min_count=2), 0)
    values = np.array([0, 1, 20], dtype=dtype)
    np.testing.assert_array_equal(nf.sigma_clipped_filter(values, maxiters=0, statistic="median", mode="wrap"), 1)
    np.testing.assert_array_equal(nf.sigma_clipped_filter(values, maxiters=0, mode="wrap"), 7)
    assert np.isnan(nf.sigma_clipped_filter(np.array([0, 0, 0, 0, 10], dtype), 5, center="mean", spread="mad",
                                            mode="wrap")).all()


def test_location_filters_literals(gpu, oracle) -> None:
    # src/location.rs:296-349 through the public filters: a window holding
    # the whole sample (wrap mode on a line of the same length, odd length).
    nf = gpu
    a = np.array([3.0, -1.5, 2.25, 8.0, 0.5, 1.75, 40.0, -6.0, 2.0, 1.0, 4.5])
    eps = np.finfo(np.float64).eps
    for got, want in ((nf.mode_filter(a, 11, mode="wrap", mode_estimator="mmm"), -4.090909090909092),
                      (nf.mode_filter(a, 11, mode="wrap"), -2.5681818181818183),
                      (nf.biweight_location_filter(a, 11, mode="wrap"), 1.9602591329467531),
                      (nf.biweight_location_filter(a, 11, mode="wrap", c=4.0), 1.8351324381177168),
                      (nf.biweight_scale_filter(a, 11, mode="wrap"), 3.281179906799965),
                      (nf.biweight_scale_filter(a, 11, mode="wrap", modify_sample_size=True), 3.128482289718106)):
        np.testing.assert_allclose(got, want, rtol=4 * eps, atol=0)
    skewed = np.array([1.0, 2.0, np.nan, 3.0, 10.0])
    np.testing.assert_array_equal(nf.nanmode_filter(skewed, 5, mode="wrap"), 2.5)
    np.testing.assert_array_equal(nf.nanmode_filter(skewed, 5, mode="wrap", mode_estimator="mmm"), -0.5)
    assert np.isnan(nf.mode_filter(skewed, 5, mode="wrap")).all()
    np.testing.assert_array_equal(nf.nanbiweight_location_filter(np.array([1.0, 2.0, 3.0, np.nan]), 4, mode="wrap"),
                                  2.0)
    assert np.isnan(nf.nanbiweight_scale_filter(np.array([1.0, 2.0, -np.inf]), 3, mode="wrap")).all()


def test_robust_validation(gpu) -> None:
    # tests/test_robust.py:339-400 (parameter checks before device work)
    nf = gpu
    x = np.zeros((0, 3))
    with pytest.raises(ValueError):
        nf.mad_filter(x, scale=-1.0)
    with pytest.raises(TypeError):
        nf.mad_filter(x, scale=True)
    with pytest.raises(ValueError):
        nf.sigma_clipped_filter(x, sigma=-1)
    with pytest.raises(ValueError):
        nf.sigma_clipped_filter(x, center="mode")
    with pytest.raises(ValueError):
        nf.sigma_clipped_filter(x, maxiters=-1)
    with pytest.raises(TypeError):
        nf.sigma_clipped_filter(x, maxiters=True)
    with pytest.raises(ValueError):
        nf.mode_filter(x, mode_estimator="median")
    with pytest.raises(ValueError):
        nf.mode_filter(x, pearson=0.5)
    with pytest.raises(ValueError):
        nf.biweight_location_filter(x, c=0.0)
    with pytest.raises(ValueError, match="min_count"):
        nf.nanmad_filter(np.ones(3), 3, min_count=4)
