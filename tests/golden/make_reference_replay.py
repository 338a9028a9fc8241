"""Record the reference's own hot-path test suite as replayable calls.

The reference's Python layer (``python/ndfiltrs``) reaches native code only
through ``ndfiltrs._core``. This script runs the reference's own test files,
unchanged and in-process, with ``ndfiltrs._core`` replaced by a recording
stand-in built from this project:

* argument handling and validation are this library's own ``_core``
  (``ndfiltrs_gb300._core``: the ctypes binding and ``ndf_plan_create``'s
  checks, which run without a device), so the reference's error tests check
  this library's errors;
* the arithmetic, which needs a GPU in this library, comes from the CPU
  oracle (``oracle/``), the restatement that the GPU is tested against.

Every ``_core`` call the tests make is recorded (arguments, input, output or
the exception type) together with the outcome of each reference test. The
GPU test ``tests/test_gpu_reference_replay.py`` replays the recorded calls
through ``ndfiltrs_gb300._core`` on the device and compares with the recorded
results, so the device library gives every answer that the reference's own
assertions accepted. The reference checkout is needed only to make the
fixture:

    python tests/golden/make_reference_replay.py --reference /path/to/ndfiltrs

Writes ``tests/golden/reference_replay_v1.npz`` (every array's bytes in one
blob) and ``reference_replay_v1.json.gz`` (the array table, the calls, each
reference test's outcome and calls, deselected tests with their reasons).
"""

from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

# The reference's test files for the windowed-statistics path and the rows
# next to it (rolling mean, robust location filters, mesh background).
FILES = [
    "test_median_network.py",
    "test_histogram_median.py",
    "test_semantics.py",
    "test_boundaries.py",
    "test_reducers_contract.py",
    "test_statistics.py",
    "test_mean.py",
    "test_robust.py",
    "test_footprint.py",
    "test_properties.py",
    "test_layout.py",
    "test_api.py",
    "test_reference.py",
    "test_rolling_mean.py",
    "test_location_filters.py",
    "test_background.py",
]

# Tests left out, each with its reason (test-id prefixes).
DESELECT = {
    "test_footprint.py::test_footprint_output_is_bitwise_identical_across_thread_counts":
        "starts fresh interpreters, which import the reference's own compiled _core",
    "test_footprint.py::test_fixpix_median_footprint_uses_unmasked_samples":
        "pixel repair (_core.fixpix_median), outside the windowed-statistics path",
    "test_location_filters.py::test_fixpix":
        "pixel repair (_core.fixpix_mean), outside the windowed-statistics path",
    "test_mean.py::test_separable_mean_matches_direct_mean":
        "method='separable' (_core.separable_smooth), outside the windowed-statistics path",
}

MAX_RECORD_BYTES = 4 << 20  # calls whose input and outputs exceed this are not stored


def _import_file(name: str, path: Path):
    import importlib.util

    spec = importlib.util.spec_from_file_location(name, path)
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


class Recorder:
    def __init__(self) -> None:
        self.calls: list[dict] = []
        self.arrays: list[np.ndarray] = []
        self.names: dict[str, int] = {}  # content hash -> array index (each array stored once)
        self.index: dict[str, int] = {}
        self.current = ""
        self.by_test: dict[str, list[int]] = {}
        self.skipped_large = 0

    def _store(self, value) -> object:
        if isinstance(value, np.ndarray):
            layout = {}
            if not value.flags.c_contiguous:
                layout["contiguous"] = False
            if not value.flags.aligned:
                layout["aligned"] = False
            if not value.flags.writeable:
                layout["writeable"] = False
            if layout:
                return dict(self._store(np.array(value, copy=True, order="C")), **layout)
            value = np.array(value, copy=True, order="C")  # the caller may change its array later
            key = hashlib.sha256(str((value.dtype.str, value.shape)).encode() + value.tobytes()).hexdigest()
            index = self.names.get(key)
            if index is None:
                index = self.names[key] = len(self.arrays)
                self.arrays.append(value)
            return {"array": index}
        if isinstance(value, (bool, np.bool_)):
            return bool(value)
        if isinstance(value, (int, np.integer)):
            return int(value)
        if isinstance(value, (float, np.floating)):
            return {"float": float(value).hex()}
        if isinstance(value, (list, tuple)):
            return [self._store(v) for v in value]
        if value is None or isinstance(value, str):
            return value
        raise TypeError(f"cannot record {type(value)!r}")

    def record(self, function: str, args: tuple, kwargs: dict, result=None, error=None) -> None:
        digest = hashlib.sha256()
        digest.update(function.encode())
        nbytes = 0
        for value in list(args) + sorted(kwargs.items()):
            if isinstance(value, np.ndarray):
                digest.update(str((value.dtype.str, value.shape)).encode())
                digest.update(np.ascontiguousarray(value).tobytes())
                nbytes += value.nbytes
            else:
                digest.update(repr(value).encode())
        key = digest.hexdigest()
        if key in self.index:
            self.by_test.setdefault(self.current, []).append(self.index[key])
            return
        if result is not None:
            outputs = result if isinstance(result, tuple) else (result,)
            nbytes += sum(o.nbytes for o in outputs if isinstance(o, np.ndarray))
        if nbytes > MAX_RECORD_BYTES:
            self.skipped_large += 1
            return
        entry = {
            "function": function,
            "args": [self._store(v) for v in args],
            "kwargs": {k: self._store(v) for k, v in kwargs.items()},
            "test": self.current,
        }
        if error is not None:
            entry["error"] = error
        else:
            entry["result"] = self._store(result)
        self.index[key] = len(self.calls)
        self.by_test.setdefault(self.current, []).append(len(self.calls))
        self.calls.append(entry)


def make_stand_in(ours, oracle, recorder: Recorder) -> types.ModuleType:
    """A module with the reference _core's names: this library's argument
    handling and validation, the oracle's arithmetic, every call recorded."""
    no_device = 9

    def needs_device(error: BaseException) -> bool:
        return isinstance(error, RuntimeError) and "CUDA device" in str(error)

    def window_filter(array, kind, size, footprint, origin, mode, cval, omit_nan, ignore_inf, min_count,
                      parameter):
        args = (array, kind, size, footprint, origin, mode, cval, omit_nan, ignore_inf, min_count, parameter)
        try:
            result = ours.window_filter(*args)
        except Exception as error:  # noqa: BLE001
            if not needs_device(error):
                recorder.record("window_filter", args, {}, error=type(error).__name__)
                raise
            fp = None if footprint is None else np.asarray(footprint, dtype=bool).reshape(tuple(size))
            cast = float(np.float32(cval)) if array.dtype == np.float32 else float(cval)
            result = oracle.window_filter(
                array, kind, tuple(size), footprint=fp, origin=tuple(origin), mode=tuple(mode), cval=cast,
                omit_nan=omit_nan, ignore_inf=ignore_inf, min_count=min_count, parameter=parameter)
        recorder.record("window_filter", args, {}, result=result)
        return result

    def robust_filter(array, size, footprint, origin, mode, cval, kind, parameter, omit_nan, ignore_inf,
                      min_count, sigma_lower, sigma_upper, maxiters, center, spread, estimator="sex",
                      modify_sample_size=False, pearson=2.5):
        args = (array, size, footprint, origin, mode, cval, kind, parameter, omit_nan, ignore_inf, min_count,
                sigma_lower, sigma_upper, maxiters, center, spread)
        kwargs = dict(estimator=estimator, modify_sample_size=modify_sample_size, pearson=pearson)
        try:
            result = ours.robust_filter(*args, **kwargs)
        except Exception as error:  # noqa: BLE001
            if not needs_device(error):
                recorder.record("robust_filter", args, kwargs, error=type(error).__name__)
                raise
            clip = kind in ("sigma_mean", "sigma_median", "sigma_mode")
            fp = None if footprint is None else np.asarray(footprint, dtype=bool).reshape(tuple(size))
            result = oracle.robust_filter(
                array, kind, tuple(size), footprint=fp, origin=tuple(origin), mode=tuple(mode),
                cval=float(cval), omit_nan=True if clip else omit_nan, ignore_inf=True if clip else ignore_inf,
                min_count=min_count, parameter=parameter, sigma_lower=sigma_lower, sigma_upper=sigma_upper,
                maxiters=maxiters, center=center if clip else "median", spread=spread if clip else "std",
                estimator=estimator if kind in ("mode", "sigma_mode") else "sex",
                modify_sample_size=modify_sample_size, pearson=pearson)
        recorder.record("robust_filter", args, kwargs, result=result)
        return result

    def mesh_background(array, mask, box_size, filter_size, estimator, sigma_lower, sigma_upper, maxiters, center,
                        spread, statistic, mode_estimator, pearson, rms, min_valid_fraction, valid_count,
                        valid_base, fill, idw_neighbors, idw_power, filter_edge, filter_threshold, threshold_kind,
                        interpolation):
        args = (array, mask, box_size, filter_size, estimator, sigma_lower, sigma_upper, maxiters, center, spread,
                statistic, mode_estimator, pearson, rms, min_valid_fraction, valid_count, valid_base, fill,
                idw_neighbors, idw_power, filter_edge, filter_threshold, threshold_kind, interpolation)
        try:
            result = ours.mesh_background(*args)
        except Exception as error:  # noqa: BLE001
            if not needs_device(error):
                recorder.record("mesh_background", args, {}, error=type(error).__name__)
                raise
            names = ("estimator", "sigma_lower", "sigma_upper", "maxiters", "center", "spread", "statistic",
                     "mode_estimator", "pearson", "rms", "min_valid_fraction", "valid_count", "valid_base",
                     "fill", "idw_neighbors", "idw_power", "filter_edge", "filter_threshold", "threshold_kind",
                     "interpolation")
            options = dict(zip(names, args[4:]))
            result = oracle.mesh_background(array, tuple(box_size), tuple(filter_size), mask=mask, **options)
        recorder.record("mesh_background", args, {}, result=tuple(result))
        return result

    module = types.ModuleType("ndfiltrs._core")
    module.window_filter = window_filter
    module.robust_filter = robust_filter
    module.mesh_background = mesh_background
    module.get_num_threads = ours.get_num_threads

    def __getattr__(name: str):
        def out_of_scope(*args, **kwargs):
            raise NotImplementedError(f"_core.{name} is outside the windowed-statistics path")

        if name.startswith("__"):
            raise AttributeError(name)
        return out_of_scope

    module.__getattr__ = __getattr__
    del no_device
    return module


class Outcomes:
    """pytest plugin: tracks the running test and every test's outcome."""

    def __init__(self, recorder: Recorder) -> None:
        self.recorder = recorder
        self.results: dict[str, str] = {}
        self.messages: dict[str, str] = {}

    def pytest_runtest_setup(self, item) -> None:
        self.recorder.current = item.nodeid

    def pytest_runtest_logreport(self, report) -> None:
        if report.when == "call" or report.outcome != "passed":
            if report.outcome != "passed" or report.nodeid not in self.results:
                self.results[report.nodeid] = report.outcome
            if report.outcome == "failed":
                self.messages[report.nodeid] = str(report.longrepr)[-600:]


def main() -> None:
    parser = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    parser.add_argument("--reference", default=os.environ.get("NDFILTRS_REFERENCE"),
                        help="checkout of the reference project (or set NDFILTRS_REFERENCE)")
    parser.add_argument("--out", default=str(HERE / "reference_replay_v1"))
    parser.add_argument("files", nargs="*", help="reference test files (default: the hot-path set)")
    args = parser.parse_args()
    if not args.reference:
        parser.error("--reference (or NDFILTRS_REFERENCE) is required")
    reference = Path(args.reference).resolve()

    # This library's _core and the oracle, loaded by file path so that the
    # reference's own ``tests`` package is the one on sys.path.
    sys.path.append(str(ROOT))
    import ndfiltrs_gb300._core as ours  # noqa: E402

    oracle = _import_file("ndf_oracle_module", ROOT / "oracle" / "oracle.py")
    oracle.build()
    os.environ["NDF_AUTOTUNE"] = "0"

    recorder = Recorder()
    sys.modules["ndfiltrs._core"] = make_stand_in(ours, oracle, recorder)
    sys.path.insert(0, str(reference / "python"))
    sys.path.insert(0, str(reference))
    for name in [m for m in sys.modules if m == "tests" or m.startswith("tests.")]:
        del sys.modules[name]
    import ndfiltrs  # noqa: F401,E402  (the reference's Python layer over the stand-in)

    import hypothesis

    hypothesis.settings.register_profile("replay", derandomize=True, database=None, deadline=None,
                                         print_blob=False)
    hypothesis.settings.load_profile("replay")

    import pytest

    files = args.files or FILES
    plugin = Outcomes(recorder)
    deselect = []
    for prefix in DESELECT:
        deselect += ["--deselect", f"tests/{prefix}"]
    os.chdir(reference)
    code = pytest.main(["-q", "-p", "no:cacheprovider", "-p", "no:randomly", "--rootdir", str(reference),
                        "-o", "addopts=", *deselect, *[str(reference / "tests" / f) for f in files]],
                       plugins=[plugin])
    passed = sorted(k for k, v in plugin.results.items() if v == "passed")
    failed = sorted(k for k, v in plugin.results.items() if v == "failed")
    skipped = sorted(k for k, v in plugin.results.items() if v == "skipped")
    meta = {
        "description": "reference test files run in-process against ndfiltrs_gb300._core's validation "
                       "with the oracle's arithmetic; every _core call recorded for replay on the GPU",
        "files": files,
        "deselected": DESELECT,
        "pytest_exit_code": int(code),
        "passed": len(passed),
        "failed": failed,
        "failure_messages": {k: plugin.messages.get(k, "") for k in failed},
        "skipped": skipped,
        "calls_not_stored_over_4MiB": recorder.skipped_large,
        "calls": recorder.calls,
        "tests": {k: recorder.by_test.get(k, []) for k in sorted(plugin.results)},
        "outcomes": {k: plugin.results[k] for k in sorted(plugin.results)},
    }
    # Every array's bytes in one blob (each at a 16-byte aligned offset), its
    # dtype, shape and offset in the table.
    table, pieces, offset = [], [], 0
    for value in recorder.arrays:
        raw = value.tobytes()
        pad = (-len(raw)) % 16
        table.append([value.dtype.str, list(value.shape), offset])
        pieces.append(raw + b"\0" * pad)
        offset += len(raw) + pad
    meta["arrays"] = table
    out = Path(args.out)
    np.savez_compressed(out.with_suffix(".npz"), blob=np.frombuffer(b"".join(pieces), dtype=np.uint8))
    with gzip.open(out.with_suffix(".json.gz"), "wt") as handle:
        json.dump(meta, handle, separators=(",", ":"), sort_keys=True)
    print(f"{len(passed)} passed, {len(failed)} failed, {len(skipped)} skipped; "
          f"{len(recorder.calls)} calls, {len(recorder.arrays)} arrays, "
          f"{recorder.skipped_large} over the size limit")


if __name__ == "__main__":
    main()
