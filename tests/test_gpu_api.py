"""Public API semantics on the GPU: layouts, ownership, canonical NaN, signed
zeros, SciPy agreement, footprints and origins (the reference's
tests/test_layout.py, test_semantics.py, test_boundaries.py and
test_footprint.py restated)."""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu


def test_layouts_return_owned_c_arrays(gpu) -> None:
    nf = gpu
    source = np.arange(24.0, dtype=np.float64).reshape(4, 6)
    for view in (source[::-1, ::2], np.asfortranarray(source), source.T, source.copy()):
        view.flags.writeable = False
        result = nf.median_filter(view, size=1)
        np.testing.assert_array_equal(result, view)
        assert result.flags.c_contiguous and result.flags.owndata and result.flags.writeable
        assert result.base is None


def test_strided_inputs_match_and_are_not_modified(gpu) -> None:
    nf = gpu
    for dtype in (np.float32, np.float64):
        source = np.arange(80, dtype=dtype).reshape(8, 10) - 40
        source[2, :5] = [np.nan, np.inf, -np.inf, -0.0, 0.0]
        for array in (source.T, source[::-1, ::2], np.asfortranarray(source)):
            original = array.copy()
            options = dict(size=(2, 3), origin=(-1, 1), mode=("mirror", "constant"))
            for fn in (nf.median_filter, nf.nanmedian_filter):
                direct = fn(array, method="direct", **options)
                sortnet = fn(array, method="sortnet", **options)
                hist = fn(array, method="histogram", **options)
                np.testing.assert_array_equal(bits(sortnet), bits(direct))
                np.testing.assert_array_equal(bits(hist), bits(direct))
            np.testing.assert_array_equal(bits(array), bits(original))


def test_canonical_nan_and_signed_zero(gpu) -> None:
    nf = gpu
    for dtype, canonical in ((np.float32, 0x7FC00000), (np.float64, 0x7FF8000000000000)):
        propagated = nf.median_filter(np.array([np.nan], dtype=dtype), size=1)
        below = nf.nanmedian_filter(np.array([1.0, np.nan, np.nan], dtype=dtype), size=3,
                                    mode="nearest", min_count=2)
        assert bits(propagated)[0] == canonical and bits(below)[1] == canonical
    zero = nf.median_filter(np.array([-0.0, -0.0, 0.0]), size=3, mode="nearest")
    assert np.signbit(zero[1])
    midpoint = nf.nanmedian_filter(np.asarray([-0.0, 0.0, np.nan]), 3, mode="constant", cval=np.nan)
    assert bits(midpoint)[1] == 0


def test_constant_values_follow_policy(gpu) -> None:
    nf = gpu
    values = np.array([np.nan], dtype=np.float64)
    assert nf.nanmedian_filter(values, 3, mode="constant", cval=2.0, min_count=2)[0] == 2.0
    assert np.isnan(nf.nanmedian_filter(values, 3, mode="constant", cval=np.inf, ignore_inf=True)[0])


def test_scipy_median_on_finite_odd_windows(gpu) -> None:
    ndimage = pytest.importorskip("scipy.ndimage")
    nf = gpu
    for dtype in (np.float32, np.float64):
        for mode in ("reflect", "constant", "nearest", "mirror", "wrap"):
            values = np.random.default_rng(1).normal(size=(31, 37)).astype(dtype)
            expected = ndimage.median_filter(values, size=(3, 5), mode=mode, cval=-7.0)
            np.testing.assert_array_equal(nf.median_filter(values, (3, 5), mode=mode, cval=-7.0), expected)
            fp = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], dtype=bool)
            expected = ndimage.rank_filter(values, 1, footprint=fp, mode=mode, cval=1.5, origin=(1, -1))
            actual = nf.rank_filter(values, 1, footprint=fp, mode=mode, cval=1.5, origin=(1, -1))
            np.testing.assert_array_equal(actual, expected)
            for q in (0.0, 100.0):
                expected = ndimage.percentile_filter(values, q, footprint=fp, mode=mode, cval=1.5)
                actual = nf.percentile_filter(values, q, footprint=fp, mode=mode, cval=1.5)
                np.testing.assert_array_equal(actual, expected)


def test_validation_errors_before_device_work(gpu) -> None:
    nf = gpu
    with pytest.raises(ValueError, match="requires size, not footprint"):
        nf.median_filter(np.zeros((5, 5)), footprint=np.ones((3, 3)), method="histogram")
    with pytest.raises(ValueError, match="method"):
        nf.median_filter(np.zeros((5, 5)), method="boxcar")
    with pytest.raises(ValueError, match="min_count"):
        nf.nanmedian_filter(np.ones(3), size=3, min_count=4)
    with pytest.raises(NotImplementedError):
        nf.mean_filter(np.ones((5, 5)), 3, method="separable")
    with pytest.raises(ValueError, match="requires size, not footprint"):
        nf.mean_filter(np.ones((5, 5)), footprint=np.ones((2, 3)), method="boxcar")


def test_get_num_threads_is_the_host_pool_size(gpu) -> None:
    """The host pool size, as in the reference; the SM count is separate."""
    assert 1 <= gpu.get_num_threads() <= 1024
    assert gpu.device_info()["sm_count"] > 0


def test_autotuner_changes_speed_not_results(gpu, oracle) -> None:
    """With the autotuner measuring every plan (mode 2, in-memory cache), the
    chosen kernels give the same bits as the built-in choice and the oracle,
    and each key is measured once."""
    import ndfiltrs_gb300 as nf
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(3)
    image = rng.normal(1000, 10, size=(150, 170)).astype(np.float32)
    image[rng.random(image.shape) < 0.02] = np.nan
    disk = np.add.outer(np.arange(-6, 7) ** 2, np.arange(-6, 7) ** 2) <= 36
    cases = [("median", (9, 9), None), ("percentile", (15, 15), None), ("median", None, disk),
             ("std", (11, 11), None)]
    try:
        nf.set_autotune(0, "")
        baseline = []
        for kind, size, fp in cases:
            shape = fp.shape if fp is not None else size
            with _core.Plan(image.shape, np.float32, kind, shape, footprint=fp, omit_nan=True,
                            percentile=84.0, parameter=1 if kind == "std" else 0) as plan:
                baseline.append(plan.run_host(image))
        nf.set_autotune(2, "")
        assert nf.autotune_entries() == 0
        for (kind, size, fp), want in zip(cases, baseline):
            shape = fp.shape if fp is not None else size
            for _ in range(2):
                with _core.Plan(image.shape, np.float32, kind, shape, footprint=fp, omit_nan=True,
                                percentile=84.0, parameter=1 if kind == "std" else 0) as plan:
                    got = plan.run_host(image)
                np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=kind)
            if kind != "std":
                ref = oracle.window_filter(image, kind, shape, footprint=fp, omit_nan=True, q=84.0)
                np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
        # Every key with two or more candidates (here each one: the sliding
        # histogram offers several tiles for windows this small) was measured
        # once.
        measured = nf.autotune_entries()
        assert 1 <= measured <= len(cases)
        for kind, size, fp in cases:
            shape = fp.shape if fp is not None else size
            _core.Plan(image.shape, np.float32, kind, shape, footprint=fp, omit_nan=True).close()
        assert nf.autotune_entries() == measured
    finally:
        nf.set_autotune(0, "")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_tma_staging_matches_remapped_staging(gpu, oracle, dtype) -> None:
    """Interior tiles staged by one TMA copy give the same bits as the
    boundary-remapped loads, for the box, network and moments kernels, 2-D and
    3-D, every mode at the edges, shifted origins, and widths whose rows are
    not 16-byte aligned (TMA off for those)."""
    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(17)
    cases = [
        ((300, 260), "median", (5, 5), None),
        ((300, 262), "median", (5, 5), None),  # rows not 16-byte aligned for float32
        ((300, 260), "percentile", (7, 7), None),
        ((300, 260), "median", None, np.add.outer(np.arange(-4, 5) ** 2, np.arange(-4, 5) ** 2) <= 16),
        ((300, 260), "std", (9, 11), None),
        ((12, 70, 68), "median", (3, 5, 5), None),
        ((12, 70, 68), "mean", (3, 3, 5), None),
    ]
    try:
        for shape, kind, size, fp in cases:
            image = rng.normal(1000, 10, size=shape).astype(dtype)
            image[rng.random(shape) < 0.02] = np.nan
            window = fp.shape if fp is not None else size
            for mode in ("reflect", "constant", "wrap"):
                origin = tuple([1] + [-1] * (len(shape) - 1))
                kw = dict(footprint=fp, origin=origin, mode=[mode] * len(shape), cval=2.5, omit_nan=True,
                          percentile=84.0, parameter=1 if kind == "std" else 0, moments="fp64")
                results = []
                for enabled in (True, False):
                    _core.set_tma(enabled)
                    with _core.Plan(shape, dtype, kind, window, **kw) as plan:
                        results.append(plan.run_host(image))
                ubits = np.uint32 if dtype == np.float32 else np.uint64
                np.testing.assert_array_equal(results[0].view(ubits), results[1].view(ubits),
                                              err_msg=str((shape, kind, mode)))
                if kind not in ("std", "mean"):
                    ref = oracle.window_filter(image, kind, window, footprint=fp, origin=origin, mode=mode,
                                               cval=2.5, omit_nan=True, q=84.0)
                    np.testing.assert_array_equal(results[0].view(ubits), ref.view(ubits))
    finally:
        _core.set_tma(True)


def test_bounded_wait_reports_timeout(gpu) -> None:
    """A device wait that can never complete gives up after its limit and is
    reported as NDF_ERR_TIMEOUT (7); the device stays usable."""
    import ndfiltrs_gb300 as nf
    from ndfiltrs_gb300 import _core

    assert _core.selftest_wait_timeout() == 7
    image = np.arange(64.0, dtype=np.float32).reshape(8, 8)
    np.testing.assert_array_equal(nf.median_filter(image, size=1), image)
