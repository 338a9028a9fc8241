"""ctypes wrapper and build recipe for the CPU oracle (``ndf_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``. The product package never imports
this module. The oracle restates the reference's windowed-statistics hot path
(ysBach/ndfiltrs v0.2.0) on the host; see the header of ``ndf_oracle.cpp`` for
the file:line each function follows and how its parity is pinned.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "ndf_oracle.cpp"
BUILD_DIR = HERE / "_build"
LIBRARY = BUILD_DIR / "libndf_oracle.so"

KINDS = {
    "median": 0,
    "median_network": 1,
    "median_histogram": 2,
    "mean": 3,
    "mean_rolling": 4,
    "min": 5,
    "max": 6,
    "var": 7,
    "std": 8,
    "rank": 9,
    "rank_histogram": 10,
    "percentile": 11,
}
MODES = {"reflect": 0, "constant": 1, "nearest": 2, "mirror": 3, "wrap": 4}


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (no FMA contraction, portable flags)."""
    BUILD_DIR.mkdir(exist_ok=True)
    if (
        not force
        and LIBRARY.exists()
        and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime
    ):
        return LIBRARY
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(
        [
            "g++",
            "-std=c++17",
            "-O3",
            "-ffp-contract=off",
            "-fno-fast-math",
            "-fPIC",
            "-shared",
            "-pthread",
            str(SOURCE),
            "-o",
            str(tmp),
        ],
        check=True,
    )
    os.replace(tmp, LIBRARY)
    return LIBRARY


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        handle = ctypes.CDLL(str(LIBRARY))
        u64p = ctypes.POINTER(ctypes.c_uint64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        i32p = ctypes.POINTER(ctypes.c_int32)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        vp = ctypes.c_void_p
        handle.ndfo_last_error.restype = ctypes.c_char_p
        handle.ndfo_map_index.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.c_int32, i64p]
        handle.ndfo_map_index.restype = ctypes.c_int
        handle.ndfo_midpoint.argtypes = [ctypes.c_double, ctypes.c_double]
        handle.ndfo_midpoint.restype = ctypes.c_double
        handle.ndfo_interpolate.argtypes = [ctypes.c_double] * 3
        handle.ndfo_interpolate.restype = ctypes.c_double
        dptr = ctypes.POINTER(ctypes.c_double)
        handle.ndfo_mean_valid.argtypes = [dptr, ctypes.c_uint64]
        handle.ndfo_mean_valid.restype = ctypes.c_double
        handle.ndfo_dispersion_valid.argtypes = [dptr, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32]
        handle.ndfo_dispersion_valid.restype = ctypes.c_double
        handle.ndfo_percentile.argtypes = [dptr, ctypes.c_uint64, ctypes.c_double]
        handle.ndfo_percentile.restype = ctypes.c_double
        handle.ndfo_window_taps.argtypes = [
            ctypes.c_int32, u64p, u64p, u8p, i64p, i32p, i64p, ctypes.c_uint64, u64p,
        ]
        handle.ndfo_window_taps.restype = ctypes.c_int
        handle.ndfo_network_size.argtypes = [ctypes.c_uint64, ctypes.c_int32]
        handle.ndfo_network_size.restype = ctypes.c_uint64
        handle.ndfo_filter.argtypes = [
            ctypes.c_int32, ctypes.c_int32, u64p, vp, vp, u64p, u8p, i64p, i32p,
            ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double, ctypes.c_int32,
        ]
        handle.ndfo_filter.restype = ctypes.c_int
        handle.ndfo_filter_ex.argtypes = handle.ndfo_filter.argtypes + [ctypes.c_int32]
        handle.ndfo_filter_ex.restype = ctypes.c_int
        handle.ndfo_exact_moments.argtypes = [
            ctypes.c_int32, ctypes.c_int32, u64p, vp, vp, u64p, u8p, i64p, i32p,
            ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32,
        ]
        handle.ndfo_exact_moments.restype = ctypes.c_int
        robust_args = [
            ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
            ctypes.c_int32, ctypes.c_double,
        ]
        handle.ndfo_robust_values.argtypes = [ctypes.c_int32, dptr, ctypes.c_uint64] + robust_args
        handle.ndfo_robust_values.restype = ctypes.c_double
        handle.ndfo_robust_filter.argtypes = [
            ctypes.c_int32, ctypes.c_int32, u64p, vp, vp, u64p, u8p, i64p, i32p,
            ctypes.c_double, ctypes.c_int32,
        ] + robust_args + [ctypes.c_int32]
        handle.ndfo_robust_filter.restype = ctypes.c_int
        handle.ndfo_mesh_background.argtypes = [
            ctypes.c_int32, ctypes.c_int32, u64p, vp, u8p, u64p, u64p,
            ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
            ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
            ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
            ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
            vp, vp, dptr, dptr, u8p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), dptr,
            ctypes.c_int32,
        ]
        handle.ndfo_mesh_background.restype = ctypes.c_int
        _lib = handle
    return _lib


def _arr(values, ctype):
    data = (ctype * len(values))(*values)
    return data


class OracleError(RuntimeError):
    """Raised with the oracle's error code and message."""

    def __init__(self, code: int, message: str) -> None:
        super().__init__(f"oracle error {code}: {message}")
        self.code = code


def _geometry(array: np.ndarray, size, footprint, origin, mode):
    rank = array.ndim
    if footprint is not None:
        fp = np.asarray(footprint) != 0
        size = fp.shape
        fp_buf = np.ascontiguousarray(fp, dtype=np.uint8).ravel()
    else:
        if np.ndim(size) == 0:
            size = (int(size),) * rank
        fp_buf = None
    if np.ndim(origin) == 0:
        origin = (int(origin),) * rank
    if isinstance(mode, str):
        mode = (mode,) * rank
    return (
        _arr([int(v) for v in array.shape], ctypes.c_uint64),
        _arr([int(v) for v in size], ctypes.c_uint64),
        fp_buf,
        _arr([int(v) for v in origin], ctypes.c_int64),
        _arr([MODES[m] for m in mode], ctypes.c_int32),
    )


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def window_filter(
    array: np.ndarray,
    kind: str,
    size=3,
    *,
    footprint=None,
    origin=0,
    mode="reflect",
    cval: float = 0.0,
    omit_nan: bool = False,
    ignore_inf: bool = False,
    min_count: int = 1,
    parameter: int = 0,
    q: float = 50.0,
    threads: int | None = None,
    direct: bool = False,
) -> np.ndarray:
    """Run one reduction of the CPU restatement over a C-contiguous array.

    Rectangular minimum / maximum and rolling means take the reference's
    separable passes unless ``direct`` asks for a traversal of every window.
    """
    array = np.ascontiguousarray(array)
    if array.dtype not in (np.float32, np.float64):
        raise TypeError("oracle input must be float32 or float64")
    shape, sz, fp, org, modes = _geometry(array, size, footprint, origin, mode)
    out = np.empty_like(array)
    fp_ptr = (
        fp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if fp is not None else None
    )
    rc = lib().ndfo_filter_ex(
        0 if array.dtype == np.float32 else 1,
        array.ndim,
        shape,
        array.ctypes.data_as(ctypes.c_void_p),
        out.ctypes.data_as(ctypes.c_void_p),
        sz,
        fp_ptr,
        org,
        modes,
        float(cval),
        KINDS[kind],
        int(bool(omit_nan)),
        int(bool(ignore_inf)),
        int(min_count),
        int(parameter),
        float(q),
        int(threads or default_threads()),
        int(bool(direct)),
    )
    if rc != 0:
        raise OracleError(rc, lib().ndfo_last_error().decode())
    return out


ROBUST_KINDS = {
    "percentile": 0,
    "mad": 1,
    "mode": 2,
    "biweight_location": 3,
    "biweight_scale": 4,
    "sigma_mean": 5,
    "sigma_median": 6,
    "sigma_mode": 7,
}
ESTIMATORS = {"sex": 0, "mmm": 1, "iraf": 2}


def _robust_args(omit_nan, ignore_inf, min_count, parameter, sigma_lower, sigma_upper, maxiters,
                 center, spread, estimator, modify_sample_size, pearson):
    return (
        int(bool(omit_nan)), int(bool(ignore_inf)), int(min_count), float(parameter),
        float(sigma_lower), float(sigma_upper), -1 if maxiters is None else int(maxiters),
        {"mean": 0, "median": 1}[center], {"std": 0, "mad": 1}[spread], ESTIMATORS[estimator],
        int(bool(modify_sample_size)), float(pearson),
    )


def robust_values(kind: str, values, *, omit_nan=False, ignore_inf=False, min_count=1,
                  parameter=0.0, sigma_lower=3.0, sigma_upper=3.0, maxiters=5, center="median",
                  spread="std", estimator="sex", modify_sample_size=False, pearson=2.5) -> float:
    """One robust reduction of a float64 sample (RobustReduction::finish)."""
    data = np.ascontiguousarray(values, dtype=np.float64)
    return lib().ndfo_robust_values(
        ROBUST_KINDS[kind], data.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), data.size,
        *_robust_args(omit_nan, ignore_inf, min_count, parameter, sigma_lower, sigma_upper, maxiters,
                      center, spread, estimator, modify_sample_size, pearson))


def robust_filter(array: np.ndarray, kind: str, size=3, *, footprint=None, origin=0, mode="reflect",
                  cval=0.0, omit_nan=False, ignore_inf=False, min_count=1, parameter=0.0,
                  sigma_lower=3.0, sigma_upper=3.0, maxiters=5, center="median", spread="std",
                  estimator="sex", modify_sample_size=False, pearson=2.5,
                  threads: int | None = None) -> np.ndarray:
    """robust_into over a C-contiguous array (src/robust.rs:725-785)."""
    array = np.ascontiguousarray(array)
    if array.dtype not in (np.float32, np.float64):
        raise TypeError("oracle input must be float32 or float64")
    shape, sz, fp, org, modes = _geometry(array, size, footprint, origin, mode)
    out = np.empty_like(array)
    fp_ptr = fp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if fp is not None else None
    rc = lib().ndfo_robust_filter(
        0 if array.dtype == np.float32 else 1, array.ndim, shape,
        array.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p), sz, fp_ptr,
        org, modes, float(cval), ROBUST_KINDS[kind],
        *_robust_args(omit_nan, ignore_inf, min_count, parameter, sigma_lower, sigma_upper, maxiters,
                      center, spread, estimator, modify_sample_size, pearson),
        int(threads or default_threads()))
    if rc != 0:
        raise OracleError(rc, lib().ndfo_last_error().decode())
    return out


MESH_DEFAULTS = dict(
    estimator="sextractor", sigma_lower=3.0, sigma_upper=3.0, maxiters=10, center="median", spread="std",
    statistic="mode", mode_estimator="sex", pearson=2.5, rms="std", min_valid_fraction=0.5,
    valid_count="finite", valid_base="mesh", fill="nearest", idw_neighbors=10, idw_power=1.0,
    filter_edge="shrink", filter_threshold=None, threshold_kind="deviation", interpolation="spline",
)


def mesh_background(data: np.ndarray, box_size, filter_size=3, mask=None, threads: int | None = None, **options):
    """MeshBackground::new + estimate + interpolate_into (src/background.rs).

    Returns (background, rms, mesh_background, mesh_rms, mesh_valid,
    mesh_finite_count, mesh_retained_count, global_background, global_rms)
    like the reference's ``_core.mesh_background``.
    """
    o = dict(MESH_DEFAULTS, **options)
    data = np.ascontiguousarray(data)
    ndim = data.ndim
    boxes = (int(box_size),) * ndim if np.ndim(box_size) == 0 else tuple(int(b) for b in box_size)
    filters = (int(filter_size),) * ndim if np.ndim(filter_size) == 0 else tuple(int(f) for f in filter_size)
    mesh_shape = tuple(-(-n // b) for n, b in zip(data.shape, boxes)) if all(b > 0 for b in boxes) else data.shape
    background = np.empty_like(data)
    rms = np.empty_like(data)
    mb = np.empty(mesh_shape, np.float64)
    mr = np.empty(mesh_shape, np.float64)
    mv = np.empty(mesh_shape, np.uint8)
    fc = np.empty(mesh_shape, np.int64)
    rc_ = np.empty(mesh_shape, np.int64)
    globals_ = np.empty(2, np.float64)
    flags = None if mask is None else np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8)
    threshold = o["filter_threshold"]
    kind = 0 if threshold is None else {"deviation": 1, "above": 2}[o["threshold_kind"]]
    pointer = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
    rc = lib().ndfo_mesh_background(
        0 if data.dtype == np.float32 else 1, ndim, _arr([int(v) for v in data.shape], ctypes.c_uint64),
        data.ctypes.data_as(ctypes.c_void_p), None if flags is None else pointer(flags, ctypes.c_uint8),
        _arr(list(boxes), ctypes.c_uint64), _arr(list(filters), ctypes.c_uint64),
        {"sextractor": 0, "sigma_clip": 1}[o["estimator"]], float(o["pearson"]), float(o["sigma_lower"]),
        float(o["sigma_upper"]), -1 if o["maxiters"] is None else int(o["maxiters"]),
        {"mean": 0, "median": 1}[o["center"]], {"std": 0, "mad": 1}[o["spread"]],
        {"mean": 0, "median": 1, "mode": 2}[o["statistic"]], ESTIMATORS[o["mode_estimator"]],
        {"std": 0, "mad": 1}[o["rms"]], float(o["min_valid_fraction"]),
        {"finite": 0, "retained": 1}[o["valid_count"]], {"mesh": 0, "box": 1}[o["valid_base"]],
        {"nearest": 0, "idw": 1}[o["fill"]], int(o["idw_neighbors"]), float(o["idw_power"]),
        {"shrink": 0, "truncate": 1}[o["filter_edge"]], kind, 0.0 if threshold is None else float(threshold),
        {"spline": 0, "sextractor": 1}[o["interpolation"]],
        background.ctypes.data_as(ctypes.c_void_p), rms.ctypes.data_as(ctypes.c_void_p),
        pointer(mb, ctypes.c_double), pointer(mr, ctypes.c_double), pointer(mv, ctypes.c_uint8),
        pointer(fc, ctypes.c_int64), pointer(rc_, ctypes.c_int64), pointer(globals_, ctypes.c_double),
        int(threads or default_threads()))
    if rc != 0:
        raise OracleError(rc, lib().ndfo_last_error().decode())
    return (background, rms, mb, mr, mv.astype(bool), fc, rc_, float(globals_[0]), float(globals_[1]))


def exact_moments(
    array: np.ndarray,
    kind: str,
    size=3,
    *,
    footprint=None,
    origin=0,
    mode="reflect",
    cval: float = 0.0,
    omit_nan: bool = False,
    ignore_inf: bool = False,
    min_count: int = 1,
    ddof: int = 0,
    threads: int | None = None,
) -> np.ndarray:
    """Exact (double-double) window mean/var/std rounded once to float64."""
    array = np.ascontiguousarray(array)
    shape, sz, fp, org, modes = _geometry(array, size, footprint, origin, mode)
    out = np.empty(array.shape, dtype=np.float64)
    fp_ptr = (
        fp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if fp is not None else None
    )
    rc = lib().ndfo_exact_moments(
        0 if array.dtype == np.float32 else 1,
        array.ndim,
        shape,
        array.ctypes.data_as(ctypes.c_void_p),
        out.ctypes.data_as(ctypes.c_void_p),
        sz,
        fp_ptr,
        org,
        modes,
        float(cval),
        KINDS[kind],
        int(bool(omit_nan)),
        int(bool(ignore_inf)),
        int(min_count),
        int(ddof),
        int(threads or default_threads()),
    )
    if rc != 0:
        raise OracleError(rc, lib().ndfo_last_error().decode())
    return out


def map_index(index: int, length: int, mode: str) -> int | None:
    out = ctypes.c_int64(0)
    rc = lib().ndfo_map_index(int(index), int(length), MODES[mode], ctypes.byref(out))
    if rc < 0:
        raise OracleError(-rc, "cannot map an empty axis")
    return int(out.value) if rc == 1 else None


def midpoint(lower: float, upper: float) -> float:
    return lib().ndfo_midpoint(float(lower), float(upper))


def interpolate(lower: float, upper: float, fraction: float) -> float:
    return lib().ndfo_interpolate(float(lower), float(upper), float(fraction))


def _dptr(values):
    buf = np.ascontiguousarray(values, dtype=np.float64)
    return buf, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mean_valid(values) -> float:
    buf, ptr = _dptr(values)
    return lib().ndfo_mean_valid(ptr, buf.size)


def dispersion_valid(values, ddof: int, std: bool) -> float:
    buf, ptr = _dptr(values)
    return lib().ndfo_dispersion_valid(ptr, buf.size, int(ddof), int(bool(std)))


def percentile(values, q: float) -> float:
    buf, ptr = _dptr(values)
    return lib().ndfo_percentile(ptr, buf.size, float(q))


def window_taps(shape, size, footprint=None, origin=0, mode="reflect") -> np.ndarray:
    array = np.empty(shape, dtype=np.float64)
    sh, sz, fp, org, modes = _geometry(array, size, footprint, origin, mode)
    rank = len(shape)
    capacity = int(np.prod(sz[:])) * rank if fp is None else int(fp.sum()) * rank
    taps = (ctypes.c_int64 * max(capacity, 1))()
    count = ctypes.c_uint64(0)
    fp_ptr = (
        fp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)) if fp is not None else None
    )
    rc = lib().ndfo_window_taps(rank, sh, sz, fp_ptr, org, modes, taps, capacity, ctypes.byref(count))
    if rc != 0:
        raise OracleError(rc, lib().ndfo_last_error().decode())
    return np.array(taps[: count.value * rank], dtype=np.int64).reshape(count.value, rank)


def network_size(count: int, omit: bool) -> int:
    return int(lib().ndfo_network_size(int(count), int(bool(omit))))
