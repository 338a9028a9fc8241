"""The plan cache of the one-call filters (``_core._PlanCache``): repeated
calls reuse a plan, results stay those of a fresh plan, threads sharing a
plan are serialized, eviction closes plans, configuration errors are not
cached, and kernel-choice changes empty the cache."""

from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _image(shape, seed):
    rng = np.random.default_rng(seed)
    image = (100 + 10 * rng.standard_normal(shape)).astype(np.float32)
    image[rng.random(shape) < 0.01] = np.nan
    return image


def _fresh(image, size):
    from ndfiltrs_gb300 import _core

    with _core.Plan(image.shape, image.dtype, "median", (size, size), omit_nan=True) as plan:
        return plan.run_host(image)


def test_reuse_threads_and_eviction(gpu) -> None:
    from ndfiltrs_gb300 import _core

    nf = gpu
    _core.clear_plan_cache()
    images = [_image((300, 257), seed) for seed in range(6)]
    expected = [_fresh(image, 5) for image in images]
    for image, want in zip(images, expected):
        np.testing.assert_array_equal(nf.nanmedian_filter(image, 5).view(np.uint32), want.view(np.uint32))
    assert len(_core._plan_cache._plans) == 1

    results = [None] * 24
    def work(i):
        results[i] = nf.nanmedian_filter(images[i % 6], 5)
    threads = [threading.Thread(target=work, args=(i,)) for i in range(24)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, got in enumerate(results):
        np.testing.assert_array_equal(got.view(np.uint32), expected[i % 6].view(np.uint32))

    for rows in range(100, 100 + 2 * _core._plan_cache.capacity):
        nf.nanmedian_filter(_image((rows, 64), rows), 3)
    assert len(_core._plan_cache._plans) == _core._plan_cache.capacity
    np.testing.assert_array_equal(nf.nanmedian_filter(images[0], 5).view(np.uint32), expected[0].view(np.uint32))

    before = len(_core._plan_cache._plans)
    with pytest.raises(ValueError):
        nf.nanmedian_filter(images[0], 5, min_count=100)
    assert len(_core._plan_cache._plans) == before

    _core.set_autotune(1)
    assert len(_core._plan_cache._plans) == 0
    np.testing.assert_array_equal(nf.nanmedian_filter(images[1], 5).view(np.uint32), expected[1].view(np.uint32))


def test_keys_separate_configurations(gpu) -> None:
    from ndfiltrs_gb300 import _core

    nf = gpu
    _core.clear_plan_cache()
    image = _image((128, 96), 9)
    a = nf.nanmedian_filter(image, 3, mode="reflect")
    b = nf.nanmedian_filter(image, 3, mode="constant", cval=np.nan)
    c = nf.nanmedian_filter(image, 3, mode="constant", cval=np.nan)
    d = nf.nanpercentile_filter(image, 84, size=3)
    assert not np.array_equal(a, b, equal_nan=True)
    np.testing.assert_array_equal(b.view(np.uint32), c.view(np.uint32))
    assert len(_core._plan_cache._plans) == 3
    assert d.shape == image.shape


def test_outputs_do_not_alias(gpu) -> None:
    """Outputs come from pooled host buffers: a live result is never
    overwritten by a later call, and a released one is reused."""
    nf = gpu
    first, second = _image((1024, 1024), 21), _image((1024, 1024), 22)
    want_first, want_second = _fresh(first, 5), _fresh(second, 5)
    out_first = nf.nanmedian_filter(first, 5)
    out_second = nf.nanmedian_filter(second, 5)
    np.testing.assert_array_equal(out_first.view(np.uint32), want_first.view(np.uint32))
    np.testing.assert_array_equal(out_second.view(np.uint32), want_second.view(np.uint32))
    assert out_first.ctypes.data != out_second.ctypes.data
    for _ in range(3):
        out_first = nf.nanmedian_filter(first, 5)
        np.testing.assert_array_equal(out_first.view(np.uint32), want_first.view(np.uint32))
        np.testing.assert_array_equal(out_second.view(np.uint32), want_second.view(np.uint32))
