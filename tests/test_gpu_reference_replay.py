"""The reference's own hot-path test suite, replayed on the GPU.

``tests/golden/make_reference_replay.py`` ran the reference's test files
(``tests/test_median_network.py``, ``test_histogram_median.py``,
``test_semantics.py``, ``test_boundaries.py``, ``test_reducers_contract.py``,
``test_statistics.py``, ``test_mean.py``, ``test_robust.py``,
``test_footprint.py``, ``test_properties.py`` with its hypothesis examples,
``test_layout.py``, ``test_api.py``, ``test_reference.py``,
``test_rolling_mean.py``, ``test_location_filters.py``,
``test_background.py``) unchanged, through the reference's own Python layer,
with ``ndfiltrs._core`` answered by this library's validation and the CPU
oracle's arithmetic, and recorded every ``_core`` call with its result; every
test outside the deselected out-of-scope ones passed that way.

Here each recorded call goes through ``ndfiltrs_gb300._core`` on the device:

* order statistics, extrema, percentiles, rolling means, the robust family
  and the mesh background must equal the recorded result bit for bit;
* mean / var / std equal it bit for bit with the float64 moments path
  (``NDF_MOMENTS=fp64``), and with the default float32-compensated path lie
  within 2 ulp (float32 output) / 1e-12 relative (float64 output) of it;
* a call that raised must raise the same exception type.

So the device library returns, for every input the reference's tests use,
the answer those tests' assertions accepted.
"""

from __future__ import annotations

import gzip
import json
import math
from collections import defaultdict
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
MOMENTS = {"mean", "var", "std"}


def _fixture():
    with gzip.open(GOLDEN / "reference_replay_v1.json.gz", "rt") as handle:
        meta = json.load(handle)
    with np.load(GOLDEN / "reference_replay_v1.npz") as archive:
        blob = archive["blob"]
    arrays = []
    for dtype, shape, offset in meta["arrays"]:
        dtype = np.dtype(dtype)
        count = math.prod(shape)
        arrays.append(np.frombuffer(blob, dtype=dtype, count=count, offset=offset).reshape(shape))
    return meta, arrays


_CACHE: dict = {}


def replay_fixture():
    if not _CACHE:
        _CACHE["meta"], _CACHE["arrays"] = _fixture()
    return _CACHE["meta"], _CACHE["arrays"]


def _layout(array: np.ndarray, spec: dict) -> np.ndarray:
    """The recorded input with its recorded layout: C-contiguous unless the
    call received a strided, misaligned or read-only array."""
    out = np.array(array, copy=True)
    if spec.get("contiguous") is False and out.ndim > 0 and out.size > 1:
        wide = np.empty(out.shape + (2,), dtype=out.dtype)
        wide[..., 0] = out
        out = wide[..., 0]
    if spec.get("aligned") is False:
        raw = np.empty(out.nbytes + 1, dtype=np.uint8)
        view = np.frombuffer(raw.data, dtype=out.dtype, count=out.size, offset=1).reshape(out.shape)
        view[...] = out
        out = view
    if spec.get("writeable") is False:
        out.flags.writeable = False
    return out


def _value(stored, arrays):
    if isinstance(stored, dict):
        if "array" in stored:
            return _layout(arrays[stored["array"]], stored)
        if "float" in stored:
            return float.fromhex(stored["float"])
    if isinstance(stored, list):
        return [_value(v, arrays) for v in stored]
    return stored


def _bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    return a


def _same(actual, expected) -> bool:
    if isinstance(expected, np.ndarray):
        actual = np.asarray(actual)
        return (actual.shape == expected.shape and actual.dtype == expected.dtype
                and np.array_equal(_bits(actual), _bits(expected)))
    if isinstance(expected, float):
        return (math.isnan(expected) and math.isnan(actual)) or float(actual) == expected
    return actual == expected


def _close_moments(actual: np.ndarray, expected: np.ndarray) -> bool:
    """Within the float32-compensated contract: 2 ulp for float32 output,
    1e-12 relative for float64 output; NaN where and only where expected."""
    actual = np.asarray(actual)
    if actual.shape != expected.shape or actual.dtype != expected.dtype:
        return False
    nan_a, nan_e = np.isnan(actual), np.isnan(expected)
    if not np.array_equal(nan_a, nan_e):
        return False
    keep = ~nan_e
    a, e = actual[keep].astype(np.float64), expected[keep].astype(np.float64)
    if not np.array_equal(np.isinf(a), np.isinf(e)) or not np.array_equal(a[np.isinf(e)], e[np.isinf(e)]):
        return False
    finite = np.isfinite(e)
    a, e = a[finite], e[finite]
    if expected.dtype == np.float32:
        ulp = np.spacing(np.abs(e.astype(np.float32))).astype(np.float64)
        return bool(np.all(np.abs(a - e) <= 2 * ulp))
    return bool(np.all(np.abs(a - e) <= 1e-12 * np.abs(e) + 1e-300))


def _run(core, call, arrays):
    args = [_value(v, arrays) for v in call["args"]]
    kwargs = {k: _value(v, arrays) for k, v in call["kwargs"].items()}
    fn = getattr(core, call["function"])
    return fn(*args, **kwargs)


def _files():
    meta, _ = replay_fixture()
    return meta["files"]


def test_fixture_records_a_green_reference_suite() -> None:
    meta, arrays = replay_fixture()
    assert not meta["failed"], meta["failed"][:5]
    assert meta["passed"] > 4000 and len(meta["calls"]) > 40000
    assert all(0 <= c < len(meta["calls"]) for ids in meta["tests"].values() for c in ids)


@pytest.fixture(scope="module")
def calls_by_file():
    meta, _ = replay_fixture()
    grouped = defaultdict(list)
    for index, call in enumerate(meta["calls"]):
        grouped[call["test"].split("::")[0].split("/")[-1]].append(index)
    return grouped


@pytest.mark.gpu
@pytest.mark.parametrize("name", [
    "test_median_network.py", "test_histogram_median.py", "test_semantics.py", "test_boundaries.py",
    "test_reducers_contract.py", "test_statistics.py", "test_mean.py", "test_robust.py", "test_footprint.py",
    "test_properties.py", "test_layout.py", "test_api.py", "test_reference.py", "test_rolling_mean.py",
    "test_location_filters.py", "test_background.py",
])
def test_reference_file_replays_on_the_device(gpu, calls_by_file, monkeypatch, name) -> None:
    from ndfiltrs_gb300 import _core

    meta, arrays = replay_fixture()
    failures = []
    for index in calls_by_file.get(name, []):
        call = meta["calls"][index]
        kind = call["args"][1] if call["function"] == "window_filter" else None
        modes = ["fp64", "fp32c"] if kind in MOMENTS and "error" not in call else [None]
        for moments in modes:
            if moments:
                monkeypatch.setenv("NDF_MOMENTS", moments)
            try:
                result = _run(_core, call, arrays)
            except Exception as error:  # noqa: BLE001
                if call.get("error") != type(error).__name__:
                    failures.append((index, call["test"], moments, f"raised {type(error).__name__}: {error}"))
                continue
            finally:
                monkeypatch.delenv("NDF_MOMENTS", raising=False)
            if "error" in call:
                failures.append((index, call["test"], moments, f"expected {call['error']}"))
                continue
            expected = _value(call["result"], arrays)
            if call["function"] == "mesh_background":
                ok = len(result) == len(expected) and all(_same(a, e) for a, e in zip(result, expected))
            elif moments == "fp32c":
                ok = _close_moments(result, expected)
            else:
                ok = _same(result, expected)
            if not ok:
                failures.append((index, call["test"], moments, "result differs"))
    assert not failures, f"{len(failures)} of {len(calls_by_file.get(name, []))} calls differ: {failures[:8]}"
