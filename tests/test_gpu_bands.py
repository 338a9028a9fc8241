"""Host-buffer runs in row bands (``ndf_plan_run_host``): uploads, kernels
and downloads of successive bands overlap, and the result equals the
whole-array run bit for bit (the kernels themselves are checked against the
oracle elsewhere)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _image(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    image = (1000.0 + 20.0 * rng.standard_normal(shape)).astype(dtype)
    flat = image.reshape(-1)
    flat[rng.choice(flat.size, flat.size // 100, replace=False)] = np.nan
    flat[rng.choice(flat.size, flat.size // 500, replace=False)] = np.inf
    flat[rng.choice(flat.size, flat.size // 500, replace=False)] = 5000.0
    return image


RING = np.hypot(*np.mgrid[-4:5, -4:5]) <= 4.5
RING[3:6, 3:6] = False

# (shape, dtype, plan options, bands expected)
CASES = [
    ((2048, 2048), np.float32, dict(kind="median", size=(5, 5), omit_nan=True), True),
    ((2048, 2048), np.float32, dict(kind="median", size=(7, 7), origin=(-3, 2), mode=("nearest", "reflect"),
                                    omit_nan=True, min_count=3), True),
    ((2048, 2048), np.float32, dict(kind="percentile", size=(9, 9), footprint=RING, percentile=84.0,
                                    mode=("constant", "wrap"), cval=2.5, omit_nan=True), True),
    ((2048, 2048), np.float32, dict(kind="median_histogram", size=(65, 65), mode=("mirror", "reflect"),
                                    omit_nan=True, ignore_inf=True), True),
    ((2048, 2048), np.float32, dict(kind="min", size=(31, 31), omit_nan=True, min_count=3), True),
    ((2048, 2048), np.float32, dict(kind="mean_rolling", size=(31, 31), omit_nan=True), True),
    ((2048, 2048), np.float32, dict(kind="std", size=(9, 9), omit_nan=True, moments="fp64"), True),
    ((2048, 2048), np.float32, dict(kind="mad", size=(5, 5), omit_nan=True, robust={"parameter": 1.4826}), True),
    ((1500, 1400), np.float64, dict(kind="median", size=(3, 3), mode=("reflect", "nearest")), True),
    ((1 << 23,), np.float32, dict(kind="median", size=(9,), origin=(2,), mode=("mirror",), omit_nan=True), True),
    ((512, 96, 96), np.float32, dict(kind="median", size=(3, 5, 5), mode=("nearest", "reflect", "wrap"),
                                     omit_nan=True), True),
    # Float32-compensated moments of float32 arrays (sliding kernel).
    ((2048, 2048), np.float32, dict(kind="std", size=(9, 9), omit_nan=True, moments="fp32c"), True),
    ((2048, 2048), np.float32, dict(kind="mean", size=(31, 31), mode=("nearest", "mirror"), omit_nan=True,
                                    ignore_inf=True, moments="fp32c"), True),
    ((2048, 2048), np.float32, dict(kind="var", size=(7, 51), origin=(2, -5), omit_nan=False,
                                    moments="fp32c"), True),
    # Not banded: wrap along the first axis, float32-compensated moments of
    # float64 arrays or footprints, arrays below 16 MiB.
    ((2048, 2048), np.float32, dict(kind="median", size=(5, 5), mode=("wrap", "reflect"), omit_nan=True), False),
    ((1500, 1400), np.float64, dict(kind="std", size=(9, 9), omit_nan=True, moments="fp32c"), False),
    ((2048, 2048), np.float32, dict(kind="std", size=(9, 9), footprint=RING, omit_nan=True, moments="fp32c"), False),
    ((1024, 1024), np.float32, dict(kind="median", size=(5, 5), omit_nan=True), False),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_bands_equal_whole_array(gpu, case) -> None:
    from ndfiltrs_gb300 import _core

    shape, dtype, options, banded = CASES[case]
    plan = _core.Plan(shape, dtype, **options)
    try:
        first, second = _image(shape, dtype, 1), _image(shape, dtype, 2)
        whole_first, whole_second = plan.run_host(first), plan.run_host(second)
        plan.set_host_bands("always")
        for image, whole in ((first, whole_first), (second, whole_second), (first, whole_first)):
            out = np.full(shape, -7.0, dtype)
            plan.run_host_async(image, out)
            np.testing.assert_array_equal(out.view(np.uint8), whole.view(np.uint8))
            assert (plan.host_bands >= 2) == banded
    finally:
        plan.close()


def test_timed_choice_and_never(gpu) -> None:
    from ndfiltrs_gb300 import _core

    shape = (2048, 2048)
    plan = _core.Plan(shape, np.float32, kind="median", size=(5, 5), omit_nan=True)
    try:
        image = _image(shape, np.float32, 3)
        whole = plan.run_host(image)
        for run in range(5):
            out = np.empty(shape, np.float32)
            plan.run_host_async(image, out)
            np.testing.assert_array_equal(out.view(np.uint8), whole.view(np.uint8))
            if run < 2:
                assert plan.host_bands == 0  # the first two runs are whole-array runs
        assert plan.host_bands in (0, 8)  # kept only when the banded run was faster
        plan.set_host_bands("never")
        out = np.empty(shape, np.float32)
        plan.run_host_async(image, out)
        assert plan.host_bands == 0
        np.testing.assert_array_equal(out.view(np.uint8), whole.view(np.uint8))
        with pytest.raises(ValueError):
            plan.set_host_bands("sometimes")
    finally:
        plan.close()
