"""Pin the oracle's mesh background to the reference.

* Golden vectors (``tests/golden/mesh_v1.npz``, made by
  ``tests/golden/make_mesh_golden.py``) from the reference's own NumPy
  statement of the pipeline (``tests/_background_reference.py``) over the case
  matrix of ``tests/test_background.py:67-90``; compared as the reference
  compares its native pipeline with that statement: 1e-11 absolute for values,
  exact for counts and validity.
* Literal results of ``src/background.rs:1214-1496`` and
  ``tests/test_background.py:113-236`` (the sep 1.4.1 map samples).
"""

from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
FIELDS = ("background", "rms", "mesh_background", "mesh_rms", "mesh_valid", "mesh_finite_count",
          "mesh_retained_count", "global_background", "global_rms")
SAMPLE = 11


def golden_image(shape, seed):
    """tests/golden/make_mesh_golden.py:image (the reference's test image)."""
    rng = np.random.default_rng(seed)
    grids = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    values = 100.0 + sum(0.02 * (axis + 1) * g for axis, g in enumerate(grids))
    values = values + rng.normal(0.0, 5.0, shape)
    flat = values.reshape(-1)
    flat[rng.choice(flat.size, flat.size // 200, replace=False)] += 800.0
    flat[rng.choice(flat.size, flat.size // 300, replace=False)] = np.nan
    return values


def golden_cases():
    cases = json.loads((GOLDEN / "mesh_v1.json").read_text())
    arrays = np.load(GOLDEN / "mesh_v1.npz")
    for case in cases:
        shape, box = tuple(case["shape"]), tuple(case["box"])
        data = golden_image(shape, len(shape) + sum(box))
        mask = np.zeros(shape, dtype=bool)
        mask[tuple(slice(0, n // 3) for n in shape)] = True
        options = {k: tuple(v) if isinstance(v, list) else v for k, v in case["options"].items()}
        expected = {name: arrays[f"{name}{case['index']}"] for name in FIELDS}
        yield shape, box, options, data, mask, expected


def _call(oracle, data, box, mask=None, **options):
    options = dict(options)
    filter_size = options.pop("filter_size", 3)
    if "pearson" not in options:
        estimator = "sex" if options.get("estimator", "sextractor") == "sextractor" else options.get(
            "mode_estimator", "sex")
        options["pearson"] = 2.5 if estimator == "sex" else 3.0
    return oracle.mesh_background(data, box, filter_size, mask=mask, **options)


def test_golden_vectors(oracle) -> None:
    count = 0
    for shape, box, options, data, mask, expected in golden_cases():
        result = dict(zip(FIELDS, _call(oracle, data, box, mask, **options)))
        for name in FIELDS:
            actual = np.asarray(result[name])
            want = np.asarray(expected[name])
            if name in ("background", "rms"):
                actual = actual.reshape(-1)[::SAMPLE]
            if actual.dtype.kind in "bi":
                np.testing.assert_array_equal(actual, want, err_msg=f"{shape} {name}")
            else:
                np.testing.assert_allclose(actual, want, rtol=0, atol=1e-11, equal_nan=True,
                                           err_msg=f"{shape} {options} {name}")
        count += 1
    assert count == 9


MEAN = dict(estimator="sigma_clip", maxiters=0, statistic="mean", rms="std")


def test_spline_reproduces_planes(oracle) -> None:
    # src/background.rs:1243-1270
    for shape, boxes in (((64, 96), (16, 16)), ((12, 10, 8), (4, 5, 4)), ((30,), (6,))):
        grids = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
        data = 3.0 + sum((0.5 - 0.25 * axis) * g for axis, g in enumerate(grids))
        result = _call(oracle, data, boxes, filter_size=1, **MEAN)
        assert result[4].all()
        np.testing.assert_allclose(result[0], data, rtol=0, atol=1e-11)


def test_spline_row_literals(oracle) -> None:
    # src/background.rs:1272-1300
    row = [0.0, 8.0, 2.0, 10.0, 4.0]
    data = np.array([row[(i % 14) // 3] for i in range(2 * 14)]).reshape(2, 14)
    background = _call(oracle, data, (2, 3), filter_size=1, **MEAN)[0]
    expected = [-4.148148148148149, 0.0, 4.148148148148149, 7.185185185185186, 8.0, 6.074074074074074,
                3.2592592592592604, 2.0, 3.9259259259259274, 7.407407407407406, 10.0, 9.851851851851851,
                7.481481481481479, 4.0]
    np.testing.assert_allclose(background[0], expected, rtol=0, atol=1e-13)
    np.testing.assert_allclose(background[1], expected, rtol=0, atol=1e-13)


def test_sextractor_interpolation_literals(oracle) -> None:
    # src/background.rs:1302-1318: one mesh row is piecewise linear.
    row = [0.0, 8.0, 2.0, 10.0]
    data = np.array([row[(i % 16) // 4] for i in range(3 * 16)]).reshape(3, 16)
    background = _call(oracle, data, (4, 4), filter_size=1, interpolation="sextractor", **MEAN)[0]
    for p in range(16):
        u = (p + 0.5) / 4.0 - 0.5
        seg = min(max(math.floor(u), 0), 2)
        t = u - seg
        assert abs(background[0, p] - ((1 - t) * row[seg] + t * row[seg + 1])) < 1e-13
    with pytest.raises(oracle.OracleError):
        _call(oracle, np.ones((3, 4, 5)), (2, 2, 2), filter_size=1, interpolation="sextractor", **MEAN)
    # tests/test_background.py:203-236: samples of a map measured with sep 1.4.1.
    grid = (np.arange(30).reshape(5, 6) ** 2 % 17).astype(np.float32)
    image = grid.repeat(3, axis=0).repeat(4, axis=1)[:-1, :-1].copy()
    pixels = np.ix_([0, 3, 7, 13], [0, 5, 9, 16, 22])
    expected = np.array([[2.89116192, -6.96700048, -2.73611975, 12.78070450, 10.42677021],
                         [-3.32890677, 8.51829243, 9.71400928, 16.72304153, 2.55588579],
                         [3.01372504, 16.78385735, 10.82570934, 2.92412043, -0.31003678],
                         [12.23737526, 10.47210693, 11.82488537, 7.89339352, 7.88244104]], dtype=np.float32)
    background = _call(oracle, image, (3, 4), filter_size=1, interpolation="sextractor")[0]
    np.testing.assert_allclose(background[pixels], expected, rtol=0,
                               atol=4 * np.finfo(np.float32).eps * np.abs(expected).max())
    # tests/test_background.py:189-200
    levels = np.array([[0, 3, 1, 8, 4, 2]], dtype=np.float64)
    image = levels.repeat(8, axis=0)
    natural = _call(oracle, image, (8, 1), filter_size=1)[0]
    np.testing.assert_allclose(natural, image, rtol=0, atol=1e-13)
    legacy = _call(oracle, image, (8, 1), filter_size=1, interpolation="sextractor")[0]
    np.testing.assert_allclose(legacy[4], [0, 3, 6, 9, 12, 15])


def test_sextractor_estimator_clips_outliers(oracle) -> None:
    # src/background.rs:1320-1331
    values = np.array([*range(1, 10), 1000.0])
    result = _call(oracle, values, (10,), filter_size=1)
    assert result[2].tolist() == [5.0]
    assert abs(result[3][0] - 2.581988897471611) < 1e-14
    assert result[6].tolist() == [9] and result[5].tolist() == [10]


def test_invalid_meshes_are_filled(oracle) -> None:
    # src/background.rs:1333-1362
    data = np.arange(9, dtype=np.float64).reshape(3, 3) * 10.0
    data[0, 0] = np.nan
    mask = np.zeros((3, 3), dtype=bool)
    mask[1, 1] = True
    result = _call(oracle, data, (1, 1), mask=mask, filter_size=1, **MEAN)
    assert result[4].reshape(-1).tolist() == [False, True, True, True, False, True, True, True, True]
    assert result[2][1, 1] == 40.0 and result[2][0, 0] == 20.0

    def idw(neighbors):
        return _call(oracle, data, (1, 1), mask=mask, filter_size=1, fill="idw", idw_neighbors=neighbors,
                     idw_power=1.0, **MEAN)[2][1, 1]

    assert idw(2) == 40.0
    w = 1.0 / math.sqrt(2.0)
    assert abs(idw(5) - (160.0 + w * 160.0) / (4.0 + 3.0 * w)) < 1e-12


def test_median_filter_edges_and_thresholds(oracle) -> None:
    # src/background.rs:1364-1388
    data = np.array([1.0, 100.0, 3.0, 4.0, 5.0])

    def run(edge, kind=None, threshold=None):
        options = dict(MEAN, filter_edge=edge)
        if kind is not None:
            options.update(threshold_kind=kind, filter_threshold=threshold)
        return _call(oracle, data, (1,), filter_size=3, **options)[2].tolist()

    assert run("shrink") == [1.0, 3.0, 4.0, 4.0, 5.0]
    assert run("truncate") == [50.5, 3.0, 4.0, 4.0, 4.5]
    assert run("shrink", "deviation", 10.0) == [1.0, 3.0, 3.0, 4.0, 5.0]
    assert run("truncate", "above", 50.0) == [1.0, 3.0, 3.0, 4.0, 5.0]


def test_validity_counts_and_bases(oracle) -> None:
    # src/background.rs:1390-1407
    data = np.array([1.0, 1.0, np.nan, np.nan, 2.0, 2.0, 2.0])

    def valid(fraction, count, base):
        return _call(oracle, data, (4,), filter_size=1, min_valid_fraction=fraction, valid_count=count,
                     valid_base=base, **MEAN)[4].tolist()

    assert valid(0.5, "finite", "mesh") == [True, True]
    assert valid(0.51, "finite", "mesh") == [False, True]
    assert valid(0.9, "retained", "box") == [False, False]
    assert valid(0.75, "finite", "box") == [False, True]


@pytest.mark.parametrize("interpolation", ["spline", "sextractor"])
def test_all_invalid_constant_and_single_sample(oracle, interpolation) -> None:
    # src/background.rs:1409-1415, tests/test_background.py:113-187
    for box in (4, 8):
        result = _call(oracle, np.full((8, 8), np.nan), box, interpolation=interpolation)
        assert np.isnan(result[0]).all() and math.isnan(result[8]) and not result[4].any()
    image = np.full((3, 8), 3, dtype=np.float32)
    result = _call(oracle, image, 1, filter_size=1, interpolation=interpolation)
    assert result[7] == 3
    np.testing.assert_array_equal(result[0], image)
    np.testing.assert_array_equal(result[1], 0)
    image = np.full((10, 15), np.finfo(np.float64).max)
    result = _call(oracle, image, (3, 4), filter_size=1, interpolation=interpolation)
    assert result[4].all()
    np.testing.assert_array_equal(result[0], image)
    np.testing.assert_array_equal(result[1], 0)


def test_invalid_configurations(oracle) -> None:
    # src/background.rs:1417-1451
    with pytest.raises(oracle.OracleError):
        _call(oracle, np.ones(4), (0,), filter_size=1)
    with pytest.raises(oracle.OracleError):
        _call(oracle, np.ones(4), (2,), filter_size=2)
    for options in (dict(fill="idw", idw_neighbors=0), dict(min_valid_fraction=1.5), dict(pearson=0.5),
                    dict(filter_threshold=math.nan, threshold_kind="above")):
        with pytest.raises(oracle.OracleError):
            _call(oracle, np.ones(4), (2,), filter_size=1, **options)
