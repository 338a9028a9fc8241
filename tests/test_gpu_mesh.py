"""Mesh background on the GPU against the oracle, bit for bit, and the
reference's behavioural tests (tests/test_background.py of ysBach/ndfiltrs
v0.2.0) through the public ``mesh_background``."""

from __future__ import annotations

import math

import numpy as np
import pytest

from tests.conftest import bits
from tests.test_oracle_mesh import golden_image

pytestmark = pytest.mark.gpu

FIELDS = ("background", "rms", "mesh_background", "mesh_rms", "mesh_valid", "mesh_finite_count",
          "mesh_retained_count", "global_background", "global_rms")

PHOTUTILS = {
    "estimator": "sigma_clip", "maxiters": 10, "statistic": "mode", "mode_estimator": "sex", "rms": "std",
    "min_valid_fraction": 0.9, "valid_count": "retained", "valid_base": "box", "fill": "idw",
    "filter_edge": "truncate",
}

CASES = [
    ((150, 230), (32, 40), {}),
    ((150, 230), (32, 40), {"mode_estimator": "mmm"}),
    ((150, 230), (25, 25), PHOTUTILS),
    ((120, 90), (16, 30), {"filter_size": (3, 5), "filter_threshold": 0.5}),
    ((120, 90), (16, 30), {**PHOTUTILS, "filter_threshold": 101.0, "threshold_kind": "above"}),
    ((97,), (10,), {"filter_size": 5}),
    ((20, 18, 15), (6, 5, 4), {}),
    ((20, 18, 15), (6, 5, 4), {**PHOTUTILS, "spread": "mad", "rms": "mad"}),
    ((64, 64), (64, 64), {}),
    ((150, 230), (32, 40), {"interpolation": "sextractor"}),
    ((200, 301), (100, 101), {**PHOTUTILS, "statistic": "median", "center": "mean", "fill": "nearest"}),
    ((130, 200), (7, 9), {"estimator": "sigma_clip", "statistic": "mean", "maxiters": None, "spread": "mad",
                          "sigma_lower": 2.0, "sigma_upper": 1.0, "interpolation": "sextractor"}),
    # 5,625 meshes, a third masked: the fill runs on several host threads.
    ((600, 600), (8, 8), PHOTUTILS),
    ((600, 600), (8, 8), {"fill": "nearest", "min_valid_fraction": 0.9}),
]


def _oracle_options(options):
    options = dict(options)
    filter_size = options.pop("filter_size", 3)
    if options.get("pearson") is None:
        rule = "sex" if options.get("estimator", "sextractor") == "sextractor" else options.get(
            "mode_estimator", "sex")
        options["pearson"] = 2.5 if rule == "sex" else 3.0
    return filter_size, options


def _compare(actual, expected, context):
    for name, a, e in zip(FIELDS, actual, expected):
        a, e = np.asarray(a), np.asarray(e)
        if a.dtype.kind == "f":
            np.testing.assert_array_equal(bits(np.ascontiguousarray(a)), bits(np.ascontiguousarray(e)),
                                          err_msg=f"{context} {name}")
        else:
            np.testing.assert_array_equal(a, e, err_msg=f"{context} {name}")


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_mesh_background_matches_oracle(gpu, oracle, case, dtype) -> None:
    nf = gpu
    shape, box, options = CASES[case]
    data = golden_image(shape, len(shape) + sum(box)).astype(dtype)
    mask = np.zeros(shape, dtype=bool)
    mask[tuple(slice(0, n // 3) for n in shape)] = True
    result = nf.mesh_background(data, box, mask=mask, **options)
    filter_size, oracle_options = _oracle_options(options)
    expected = oracle.mesh_background(data, box, filter_size, mask=mask, **oracle_options)
    _compare(result, expected, (shape, box, options))
    assert result.background.dtype == dtype and result.mesh_background.dtype == np.float64


def test_large_meshes_use_global_scratch(gpu, oracle) -> None:
    """Meshes of 128 x 100 samples (beyond the shared-memory sort buffer)."""
    nf = gpu
    data = golden_image((300, 260), 9)
    result = nf.mesh_background(data, (128, 100))
    expected = oracle.mesh_background(data, (128, 100), 3)
    _compare(result, expected, "large meshes")


def test_reference_behaviour(gpu) -> None:
    nf = gpu
    # tests/test_background.py:113-121
    for interpolation in ("spline", "sextractor"):
        for box in (4, 8):
            r = nf.mesh_background(np.full((8, 8), np.nan), box, interpolation=interpolation)
            assert np.isnan(r.background).all() and math.isnan(r.global_rms) and not r.mesh_valid.any()
        # tests/test_background.py:169-187
        image = np.full((3, 8), 3, dtype=np.float32)
        r = nf.mesh_background(image, 1, filter_size=1, interpolation=interpolation)
        assert r.global_background == 3
        np.testing.assert_array_equal(r.background, image)
        np.testing.assert_array_equal(r.rms, 0)
        image = np.full((10, 15), np.finfo(np.float64).max)
        r = nf.mesh_background(image, (3, 4), filter_size=1, interpolation=interpolation)
        assert r.mesh_valid.all()
        np.testing.assert_array_equal(r.background, image)
    # tests/test_background.py:189-200
    levels = np.array([[0, 3, 1, 8, 4, 2]], dtype=np.float64)
    image = levels.repeat(8, axis=0)
    np.testing.assert_allclose(nf.mesh_background(image, (8, 1), filter_size=1).background, image, rtol=0,
                               atol=1e-13)
    legacy = nf.mesh_background(image, (8, 1), filter_size=1, interpolation="sextractor")
    np.testing.assert_allclose(legacy.background[4], [0, 3, 6, 9, 12, 15])
    # tests/test_background.py:203-236: samples of a sep 1.4.1 map.
    grid = (np.arange(30).reshape(5, 6) ** 2 % 17).astype(np.float32)
    image = grid.repeat(3, axis=0).repeat(4, axis=1)[:-1, :-1].copy()
    expected = np.array([[2.89116192, -6.96700048, -2.73611975, 12.78070450, 10.42677021],
                         [-3.32890677, 8.51829243, 9.71400928, 16.72304153, 2.55588579],
                         [3.01372504, 16.78385735, 10.82570934, 2.92412043, -0.31003678],
                         [12.23737526, 10.47210693, 11.82488537, 7.89339352, 7.88244104]], dtype=np.float32)
    r = nf.mesh_background(image, (3, 4), filter_size=1, interpolation="sextractor")
    np.testing.assert_allclose(r.background[np.ix_([0, 3, 7, 13], [0, 5, 9, 16, 22])], expected, rtol=0,
                               atol=4 * np.finfo(np.float32).eps * np.abs(expected).max())
    # tests/test_background.py:92-101 and 104-111
    image = golden_image((64, 80), 3)
    single = nf.mesh_background(image.astype(np.float32), 16)
    double = nf.mesh_background(image.astype(np.float32).astype(np.float64), 16)
    np.testing.assert_array_equal(single.mesh_background, double.mesh_background)
    np.testing.assert_array_equal(single.background, double.background.astype(np.float32))
    image = golden_image((80, 60), 4)
    mask = np.zeros(image.shape, dtype=np.uint8)
    mask[10:30, 5:25] = 7
    view = np.asfortranarray(image)[::-1]
    a = nf.mesh_background(view, 20, mask=mask[::-1])
    b = nf.mesh_background(np.ascontiguousarray(view), 20, mask=mask[::-1] != 0)
    _compare(a, b, "layout")


@pytest.mark.parametrize(("kwargs", "error"), [
    ({"box_size": 0}, ValueError), ({"box_size": (4,)}, ValueError), ({"box_size": 2.5}, TypeError),
    ({"filter_size": 2}, ValueError), ({"estimator": "histogram"}, ValueError),
    ({"min_valid_fraction": 1.5}, ValueError), ({"sigma": True}, TypeError), ({"maxiters": -1}, ValueError),
    ({"fill": "idw", "idw_neighbors": 0}, ValueError), ({"filter_threshold": np.nan}, ValueError),
    ({"mask": np.zeros((4, 4), dtype=bool)}, ValueError), ({"mask": np.zeros((8, 8), dtype=complex)}, TypeError),
    ({"interpolation": "linear"}, ValueError)])
def test_invalid_arguments(gpu, kwargs, error) -> None:
    # tests/test_background.py:124-146
    arguments = {"box_size": 4, **kwargs}
    with pytest.raises(error):
        gpu.mesh_background(np.ones((8, 8)), **arguments)
    with pytest.raises(ValueError, match="2-D"):
        gpu.mesh_background(np.ones((8, 8, 8)), 4, interpolation="sextractor")
