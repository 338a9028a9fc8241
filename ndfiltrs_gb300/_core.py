"""Native module of ndfiltrs_gb300: the GB300 replacement of ``ndfiltrs._core``.

It exposes the three functions the reference's Python layer calls on the
windowed-statistics path with the same positional signatures, argument
meaning and error classes (src/pyapi/filter.rs:261-314,378-380 and
src/pyapi/robust.rs:78-171 of ysBach/ndfiltrs v0.2.0):

* ``window_filter(array, kind, size, footprint, origin, mode, cval, omit_nan,
  ignore_inf, min_count, parameter)``
* ``robust_filter(array, size, footprint, origin, mode, cval, kind, parameter,
  omit_nan, ignore_inf, min_count, sigma_lower, sigma_upper, maxiters, center,
  spread, estimator="sex", modify_sample_size=False, pearson=2.5)``
* ``get_num_threads()``

Every call goes through the C-ABI library ``libndfiltrs_gb300.so`` (CUDA,
sm_103a). There is no CPU fallback: without the built library or a CUDA
device the calls raise.

Like the reference, the input is snapshotted (copied to the device) while
the GIL is held, and the computation runs with the GIL released.
"""

from __future__ import annotations

import collections
import ctypes
import os
import threading
from pathlib import Path

import numpy as np

from . import _build

NDF_OK = 0
_ERRORS = {
    1: ValueError,  # EmptyAxis
    2: ValueError,  # InvalidConfiguration
    3: ValueError,  # LengthMismatch
    4: MemoryError,
    5: OverflowError,
    6: RuntimeError,  # CUDA runtime failure
    7: TimeoutError,
    8: NotImplementedError,
    9: RuntimeError,  # no CUDA device
}

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
    "mad": 12,
    "mode": 13,
    "biweight_location": 14,
    "biweight_scale": 15,
    "sigma_mean": 16,
    "sigma_median": 17,
    "sigma_mode": 18,
}
ROBUST_KINDS = ("mad", "mode", "biweight_location", "biweight_scale", "sigma_mean", "sigma_median",
                "sigma_mode")
CENTERS = {"mean": 0, "median": 1}
SPREADS = {"std": 0, "mad": 1}
ESTIMATORS = {"sex": 0, "mmm": 1, "iraf": 2}
MODES = {"reflect": 0, "constant": 1, "nearest": 2, "mirror": 3, "wrap": 4}
MOMENTS = {"fp32c": 0, "fp64": 1}


class RobustParams(ctypes.Structure):
    _fields_ = [
        ("parameter", ctypes.c_double),
        ("sigma_lower", ctypes.c_double),
        ("sigma_upper", ctypes.c_double),
        ("maxiters", ctypes.c_int64),
        ("center", ctypes.c_int32),
        ("spread", ctypes.c_int32),
        ("estimator", ctypes.c_int32),
        ("modify_sample_size", ctypes.c_int32),
        ("pearson", ctypes.c_double),
    ]


class MeshConfig(ctypes.Structure):
    _fields_ = [
        ("estimator", ctypes.c_int32),
        ("pearson", ctypes.c_double),
        ("sigma_lower", ctypes.c_double),
        ("sigma_upper", ctypes.c_double),
        ("maxiters", ctypes.c_int64),
        ("center", ctypes.c_int32),
        ("spread", ctypes.c_int32),
        ("statistic", ctypes.c_int32),
        ("mode_estimator", ctypes.c_int32),
        ("rms", ctypes.c_int32),
        ("min_valid_fraction", ctypes.c_double),
        ("valid_count", ctypes.c_int32),
        ("valid_base", ctypes.c_int32),
        ("fill", ctypes.c_int32),
        ("idw_neighbors", ctypes.c_uint64),
        ("idw_power", ctypes.c_double),
        ("filter_edge", ctypes.c_int32),
        ("threshold_kind", ctypes.c_int32),
        ("threshold", ctypes.c_double),
        ("interpolation", ctypes.c_int32),
    ]


class FilterDesc(ctypes.Structure):
    """``ndf_filter_desc`` of include/ndfiltrs_gb300.h."""

    _fields_ = [
        ("dtype", ctypes.c_int32),
        ("ndim", ctypes.c_int32),
        ("shape", ctypes.POINTER(ctypes.c_uint64)),
        ("size", ctypes.POINTER(ctypes.c_uint64)),
        ("footprint", ctypes.POINTER(ctypes.c_uint8)),
        ("origin", ctypes.POINTER(ctypes.c_int64)),
        ("modes", ctypes.POINTER(ctypes.c_int32)),
        ("cval", ctypes.c_double),
        ("kind", ctypes.c_int32),
        ("omit_nan", ctypes.c_int32),
        ("ignore_inf", ctypes.c_int32),
        ("min_count", ctypes.c_uint64),
        ("parameter", ctypes.c_uint64),
        ("percentile", ctypes.c_double),
        ("moments", ctypes.c_int32),
        ("robust", ctypes.POINTER(RobustParams)),
    ]


_lock = threading.Lock()
_lib: ctypes.CDLL | None = None
_pylib: ctypes.PyDLL | None = None


def library_path() -> Path:
    return _build.LIBRARY


def _load() -> tuple[ctypes.CDLL, ctypes.PyDLL]:
    """Load the CUDA library (GIL-releasing and GIL-holding handles)."""
    global _lib, _pylib
    if _lib is not None and _pylib is not None:
        return _lib, _pylib
    with _lock:
        if _lib is None:
            path = library_path()
            if not path.exists():
                raise ImportError(
                    f"the CUDA library {path} is not built; run "
                    "`python -c 'import __graft_entry__ as g; g.build()'` or "
                    "`python -m ndfiltrs_gb300._build`"
                )
            lib = ctypes.CDLL(str(path))
            pylib = ctypes.PyDLL(str(path))
            vp = ctypes.c_void_p
            plan_p = ctypes.c_void_p
            for handle in (lib, pylib):
                handle.ndf_last_error.restype = ctypes.c_char_p
                handle.ndf_plan_create.argtypes = [ctypes.POINTER(FilterDesc), ctypes.POINTER(plan_p)]
                handle.ndf_plan_create.restype = ctypes.c_int
                handle.ndf_plan_destroy.argtypes = [plan_p]
                handle.ndf_plan_destroy.restype = ctypes.c_int
                handle.ndf_plan_run.argtypes = [plan_p, vp, vp, vp]
                handle.ndf_plan_run.restype = ctypes.c_int
                handle.ndf_plan_run_host.argtypes = [plan_p, vp, vp, vp]
                handle.ndf_plan_run_host.restype = ctypes.c_int
                handle.ndf_plan_upload.argtypes = [plan_p, vp]
                handle.ndf_plan_upload.restype = ctypes.c_int
                handle.ndf_plan_compute_download.argtypes = [plan_p, vp]
                handle.ndf_plan_compute_download.restype = ctypes.c_int
                handle.ndf_plan_algorithm.argtypes = [plan_p]
                handle.ndf_plan_algorithm.restype = ctypes.c_char_p
                handle.ndf_plan_host_bands.argtypes = [plan_p]
                handle.ndf_plan_host_bands.restype = ctypes.c_int32
                handle.ndf_plan_set_host_bands.argtypes = [plan_p, ctypes.c_int32]
                handle.ndf_plan_set_host_bands.restype = ctypes.c_int
                handle.ndf_get_num_threads.restype = ctypes.c_int32
                handle.ndf_device_info.argtypes = [
                    ctypes.POINTER(ctypes.c_int32),
                    ctypes.POINTER(ctypes.c_int32),
                    ctypes.POINTER(ctypes.c_int32),
                    ctypes.c_char_p,
                    ctypes.c_size_t,
                ]
                handle.ndf_device_info.restype = ctypes.c_int
                handle.ndf_batch_create.argtypes = [
                    ctypes.POINTER(FilterDesc),
                    ctypes.c_int32,
                    ctypes.POINTER(plan_p),
                ]
                handle.ndf_batch_create.restype = ctypes.c_int
                handle.ndf_batch_destroy.argtypes = [plan_p]
                handle.ndf_batch_destroy.restype = ctypes.c_int
                handle.ndf_batch_run.argtypes = [plan_p, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
                handle.ndf_batch_run.restype = ctypes.c_int
                handle.ndf_batch_run_host.argtypes = [plan_p, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
                handle.ndf_batch_run_host.restype = ctypes.c_int
                handle.ndf_set_autotune.argtypes = [ctypes.c_int32, ctypes.c_char_p]
                handle.ndf_set_autotune.restype = ctypes.c_int
                handle.ndf_autotune_entries.restype = ctypes.c_int32
                handle.ndf_pin_kernel.argtypes = [ctypes.c_char_p]
                handle.ndf_pin_kernel.restype = ctypes.c_int
                dp = ctypes.POINTER(ctypes.c_double)
                i64p = ctypes.POINTER(ctypes.c_int64)
                u8p = ctypes.POINTER(ctypes.c_uint8)
                u64p = ctypes.POINTER(ctypes.c_uint64)
                mesh_tail = [ctypes.POINTER(MeshConfig), vp, vp, dp, dp, u8p, i64p, i64p, dp]
                handle.ndf_mesh_background.argtypes = [vp, u8p, ctypes.c_int32, ctypes.c_int32, u64p, u64p,
                                                       u64p] + mesh_tail
                handle.ndf_mesh_background.restype = ctypes.c_int
                handle.ndf_mesh_background_device.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int32, u64p,
                                                              u64p, u64p] + mesh_tail + [vp]
                handle.ndf_mesh_background_device.restype = ctypes.c_int
                handle.ndf_set_tma.argtypes = [ctypes.c_int32]
                handle.ndf_set_tma.restype = ctypes.c_int
                handle.ndf_device_status.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
                handle.ndf_device_status.restype = ctypes.c_int
                handle.ndf_selftest_wait_timeout.restype = ctypes.c_int
                handle.ndf_batch_launches.argtypes = [plan_p]
                handle.ndf_batch_launches.restype = ctypes.c_int32
            _lib, _pylib = lib, pylib
    assert _lib is not None and _pylib is not None
    return _lib, _pylib


def _raise(code: int, lib: ctypes.CDLL) -> None:
    message = lib.ndf_last_error().decode(errors="replace")
    raise _ERRORS.get(code, RuntimeError)(message)


def _check(code: int, lib: ctypes.CDLL) -> None:
    if code != NDF_OK:
        _raise(code, lib)


def _u64(values) -> ctypes.Array:
    return (ctypes.c_uint64 * max(len(values), 1))(*[int(v) for v in values])


def _i64(values) -> ctypes.Array:
    return (ctypes.c_int64 * max(len(values), 1))(*[int(v) for v in values])


def _i32(values) -> ctypes.Array:
    return (ctypes.c_int32 * max(len(values), 1))(*[int(v) for v in values])


def _robust_params(robust: dict | None) -> RobustParams:
    """The ndf_robust_params of a robust kind's options (defaults as the
    reference's ClipConfig::new(3.0) and the estimators' defaults)."""
    options = dict(robust or {})
    maxiters = options.get("maxiters", 5)
    return RobustParams(
        float(options.get("parameter", 0.0)),
        float(options.get("sigma_lower", 3.0)),
        float(options.get("sigma_upper", 3.0)),
        -1 if maxiters is None else int(maxiters),
        CENTERS[options.get("center", "median")],
        SPREADS[options.get("spread", "std")],
        ESTIMATORS[options.get("estimator", "sex")],
        int(bool(options.get("modify_sample_size", False))),
        float(options.get("pearson", 2.5)),
    )


class _Lease:
    """The owner of one pooled host buffer while arrays view it: numpy keeps
    it as their base, and its finalizer returns the buffer to the pool."""

    __slots__ = ("raw", "pool", "__array_interface__")

    def __init__(self, raw: np.ndarray, pool: "_HostBuffers", shape: tuple, dtype: np.dtype) -> None:
        self.raw = raw
        self.pool = pool
        self.__array_interface__ = {"data": (raw.ctypes.data, False), "shape": tuple(shape),
                                    "typestr": np.dtype(dtype).str, "version": 3}

    def __del__(self) -> None:
        try:
            self.pool.give_back(self.raw)
        except Exception:  # interpreter shutdown
            pass


class _HostBuffers:
    """Host buffers for the output arrays of host-buffer runs. A fresh
    output array's pages are mapped one fault at a time as the device copy
    writes them, which costs more than the filter on large arrays; outputs
    are therefore views of pooled buffers whose pages are already resident,
    and a buffer returns to the pool when the last array viewing it is
    released (a loop that drops each frame's result reuses two buffers).
    Every element of an output is written by the filter. Idle buffers are
    kept up to ``max_idle_bytes``; arrays under 1 MiB are plain numpy
    allocations."""

    def __init__(self, max_idle_bytes: int = 2 << 30) -> None:
        self.max_idle_bytes = max_idle_bytes
        self._free: dict = {}
        self._idle = 0
        # Guards _free and _idle: a lease's finalizer can run on any thread at
        # any garbage-collection point. give_back never re-enters the pool, so
        # taking the lock there cannot deadlock.
        self._lock = threading.Lock()

    def array(self, shape: tuple, dtype: np.dtype) -> np.ndarray:
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
        if nbytes < (1 << 20):
            return np.zeros(shape, dtype=dtype)
        raw = None
        with self._lock:
            queue = self._free.get(nbytes)
            if queue:
                raw = queue.popleft()
                self._idle -= nbytes
        if raw is None:
            raw = np.empty(nbytes, np.uint8)
        return np.asarray(_Lease(raw, self, shape, dtype))

    def give_back(self, raw: np.ndarray) -> None:
        with self._lock:
            if self._idle + raw.nbytes > self.max_idle_bytes:
                return
            self._free.setdefault(raw.nbytes, collections.deque()).append(raw)
            self._idle += raw.nbytes


_host_buffers = _HostBuffers()


class Plan:
    """A validated filter plan (``WindowFilter::new``, src/plan.rs:260-324).

    The plan keeps its device tables and, for host-buffer runs, its device
    input/output buffers until it is closed.
    """

    def __init__(
        self,
        shape,
        dtype,
        kind: str,
        size,
        footprint=None,
        origin=None,
        mode=None,
        cval: float = 0.0,
        omit_nan: bool = False,
        ignore_inf: bool = False,
        min_count: int = 1,
        parameter: int = 0,
        percentile: float = 50.0,
        moments: str | None = None,
        robust: dict | None = None,
    ) -> None:
        lib, _ = _load()
        shape = tuple(int(v) for v in shape)
        ndim = len(shape)
        dtype = np.dtype(dtype)
        if dtype not in (np.float32, np.float64):
            raise TypeError("array dtype must be float32 or float64")
        size = list(size)
        origin = [0] * ndim if origin is None else list(origin)
        mode = ["reflect"] * ndim if mode is None else list(mode)
        if len(size) != ndim or len(origin) != ndim or len(mode) != ndim:
            raise ValueError("array, window, origin, and mode must have equal rank")
        modes = []
        for name in mode:
            if name not in MODES:
                raise ValueError("unsupported boundary mode")
            modes.append(MODES[name])
        if kind not in KINDS:
            raise ValueError("unsupported window filter kind")
        self._keep = []
        volume = 1
        for value in size:
            volume *= int(value)
        fp_ptr = None
        if footprint is not None:
            mask = np.ascontiguousarray(np.asarray(footprint, dtype=bool).ravel(), dtype=np.uint8)
            if mask.size != volume:
                raise ValueError("input length does not match the configured shape")
            self._keep.append(mask)
            fp_ptr = mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        if moments is None:
            import os

            moments = os.environ.get("NDF_MOMENTS", "fp32c")
        if moments not in MOMENTS:
            raise ValueError("moments must be 'fp32c' or 'fp64'")
        shape_a, size_a, origin_a, modes_a = _u64(shape), _u64(size), _i64(origin), _i32(modes)
        self._keep += [shape_a, size_a, origin_a, modes_a]
        desc = FilterDesc(
            0 if dtype == np.float32 else 1,
            ndim,
            shape_a,
            size_a,
            fp_ptr,
            origin_a,
            modes_a,
            float(cval),
            KINDS[kind],
            int(bool(omit_nan)),
            int(bool(ignore_inf)),
            int(min_count),
            int(parameter),
            float(percentile),
            MOMENTS[moments],
            None,
        )
        if kind in ROBUST_KINDS:
            params = _robust_params(robust)
            self._keep.append(params)
            desc.robust = ctypes.pointer(params)
        handle = ctypes.c_void_p()
        _check(lib.ndf_plan_create(ctypes.byref(desc), ctypes.byref(handle)), lib)
        self._handle = handle
        self.shape = shape
        self.dtype = dtype
        self.kind = kind

    @property
    def algorithm(self) -> str:
        lib, _ = _load()
        return lib.ndf_plan_algorithm(self._handle).decode()

    @property
    def is_open(self) -> bool:
        return getattr(self, "_handle", None) is not None and bool(self._handle.value)

    @property
    def host_bands(self) -> int:
        """Row bands ``run_host_async`` pipelines (0: the whole array at once)."""
        lib, _ = _load()
        return int(lib.ndf_plan_host_bands(self._handle))

    def set_host_bands(self, mode: str) -> None:
        """Band policy of ``run_host_async``: 'never', 'timed' (default: tried
        on the third run, kept when faster) or 'always' (where bands apply)."""
        lib, _ = _load()
        modes = {"never": 0, "timed": 1, "always": 2}
        if mode not in modes:
            raise ValueError("band mode must be 'never', 'timed' or 'always'")
        _check(lib.ndf_plan_set_host_bands(self._handle, modes[mode]), lib)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._handle

    def _check_array(self, array: np.ndarray) -> None:
        if array.shape != self.shape or array.dtype != self.dtype:
            raise ValueError("input length does not match the configured shape")

    def run_host(self, array: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        """Snapshot ``array`` to the device under the GIL, filter, copy back."""
        lib, pylib = _load()
        self._check_array(array)
        if not array.flags.c_contiguous:
            raise ValueError("native input must be C-contiguous")
        if out is None:
            out = np.zeros(self.shape, dtype=self.dtype) if array.size == 0 else _host_buffers.array(self.shape, self.dtype)
        if array.size == 0:
            return out
        _check(pylib.ndf_plan_upload(self._handle, array.ctypes.data), lib)
        _check(lib.ndf_plan_compute_download(self._handle, out.ctypes.data), lib)
        return out

    def run_host_async(self, array: np.ndarray, out: np.ndarray, stream: int = 0) -> None:
        """H2D + kernel + D2H on ``stream`` (synchronized before returning)."""
        lib, _ = _load()
        _check(lib.ndf_plan_run_host(self._handle, array.ctypes.data, out.ctypes.data, stream), lib)

    def run_device(self, d_in: int, d_out: int, stream: int = 0) -> None:
        """Enqueue the filter over device pointers on ``stream``."""
        lib, _ = _load()
        _check(lib.ndf_plan_run(self._handle, d_in, d_out, stream), lib)

    def close(self) -> None:
        if getattr(self, "_handle", None) is not None and self._handle.value:
            lib, _ = _load()
            lib.ndf_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "Plan":
        return self

    def __exit__(self, *exc) -> None:
        self.close()


class Batch:
    """Batched persistent path over many float32 images (``ndf_batch_*``).

    ``specs`` is a list of dicts with the Plan keyword arguments (``shape``,
    ``kind``, ``size``, ``footprint``, ``origin``, ``mode``, ``cval``,
    ``omit_nan``, ``ignore_inf``, ``min_count``, ``parameter``,
    ``percentile``, ``moments``, and ``robust`` for the robust kinds).
    ``run_device`` takes device pointers of
    every image and enqueues the captured CUDA graph on ``stream``.
    """

    def __init__(self, specs: list[dict]) -> None:
        lib, _ = _load()
        self._keep = []
        descs = (FilterDesc * len(specs))()
        for i, spec in enumerate(specs):
            shape = tuple(int(v) for v in spec["shape"])
            ndim = len(shape)
            footprint = spec.get("footprint")
            size = list(np.asarray(footprint).shape) if footprint is not None else list(spec["size"])
            origin = list(spec.get("origin") or [0] * ndim)
            mode = spec.get("mode") or ["reflect"] * ndim
            if isinstance(mode, str):
                mode = [mode] * ndim
            fp_ptr = None
            if footprint is not None:
                mask = np.ascontiguousarray(np.asarray(footprint, dtype=bool).ravel(), dtype=np.uint8)
                self._keep.append(mask)
                fp_ptr = mask.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            arrays = (_u64(shape), _u64(size), _i64(origin), _i32([MODES[m] for m in mode]))
            self._keep.append(arrays)
            descs[i] = FilterDesc(
                0, ndim, arrays[0], arrays[1], fp_ptr, arrays[2], arrays[3],
                float(np.float32(spec.get("cval", 0.0))), KINDS[spec["kind"]],
                int(bool(spec.get("omit_nan", False))), int(bool(spec.get("ignore_inf", False))),
                int(spec.get("min_count", 1)), int(spec.get("parameter", 0)),
                float(spec.get("percentile", 50.0)), MOMENTS[spec.get("moments", "fp32c")],
            )
            if spec["kind"] in ROBUST_KINDS:
                params = _robust_params(spec.get("robust"))
                self._keep.append(params)
                descs[i].robust = ctypes.pointer(params)
        handle = ctypes.c_void_p()
        _check(lib.ndf_batch_create(descs, len(specs), ctypes.byref(handle)), lib)
        self._handle = handle
        self.count = len(specs)
        self._shapes = [tuple(int(v) for v in spec["shape"]) for spec in specs]

    @property
    def launches(self) -> int:
        lib, _ = _load()
        return int(lib.ndf_batch_launches(self._handle))

    def run_device(self, d_in: list[int], d_out: list[int], stream: int = 0) -> None:
        lib, _ = _load()
        if len(d_in) != self.count or len(d_out) != self.count:
            raise ValueError("one input and one output pointer per image")
        ins = (ctypes.c_void_p * self.count)(*d_in)
        outs = (ctypes.c_void_p * self.count)(*d_out)
        _check(lib.ndf_batch_run(self._handle, ins, outs, stream), lib)

    def run_host(self, images: list, outputs: list | None = None) -> list:
        """Filter host arrays (float32, C-contiguous, one per spec) through
        the batch's host pipeline and return the results (new arrays unless
        ``outputs`` is given)."""
        lib, _ = _load()
        if len(images) != self.count:
            raise ValueError("one input array per image")
        arrays = []
        for image, shape in zip(images, self._shapes):
            array = np.asarray(image)
            if array.dtype != np.float32 or array.shape != shape:
                raise ValueError("batched images must be float32 arrays of the planned shapes")
            arrays.append(np.ascontiguousarray(array))
        if outputs is None:
            outputs = [np.empty(shape, dtype=np.float32) for shape in self._shapes]
        elif len(outputs) != self.count or any(
                o.dtype != np.float32 or o.shape != s or not o.flags.c_contiguous
                for o, s in zip(outputs, self._shapes)):
            raise ValueError("outputs must be C-contiguous float32 arrays of the planned shapes")
        ins = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in arrays])
        outs = (ctypes.c_void_p * self.count)(*[o.ctypes.data for o in outputs])
        _check(lib.ndf_batch_run_host(self._handle, ins, outs, None), lib)
        return outputs

    def close(self) -> None:
        if getattr(self, "_handle", None) is not None and self._handle.value:
            lib, _ = _load()
            lib.ndf_batch_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


class _PlanCache:
    """Plans of recent one-call filters, reused by later calls with the same
    configuration. Creating a plan validates it, uploads its window tables,
    picks and sizes its kernels and allocates its device buffers, which
    costs more than filtering a small array; pipelines that filter many
    frames of one shape pay it once. Least recently used plans are closed
    beyond ``capacity`` plans or ``max_bytes`` of their device buffers. A
    lock per plan serializes the calls that share it; changing the kernel
    choice rules (``set_autotune``, ``pin_kernel``) empties the cache."""

    def __init__(self, capacity: int = 8, max_bytes: int = 4 << 30) -> None:
        self.capacity = capacity
        self.max_bytes = max_bytes
        self._lock = threading.Lock()
        self._plans: collections.OrderedDict = collections.OrderedDict()

    def _evict_locked(self) -> list:
        """Remove the entries beyond the limits (the cache lock is held) and
        return them; the caller closes them after releasing the cache lock,
        so a long filter on an evicted plan never blocks other lookups."""
        evicted = []
        while self._plans and (len(self._plans) > self.capacity
                               or sum(e[2] for e in self._plans.values()) > self.max_bytes):
            evicted.append(self._plans.popitem(last=False)[1])
        return evicted

    @staticmethod
    def _close(entries) -> None:
        for plan, lock, _ in entries:
            with lock:
                plan.close()

    def run(self, key, make, array: np.ndarray) -> np.ndarray:
        with self._lock:
            entry = self._plans.get(key)
            if entry is not None:
                self._plans.move_to_end(key)
        if entry is None:
            plan = make()  # a configuration error raises here; nothing is cached
            evicted = []
            with self._lock:
                entry = self._plans.get(key)
                if entry is None:
                    entry = (plan, threading.Lock(), 2 * array.nbytes)
                    self._plans[key] = entry
                    evicted = self._evict_locked()
            if entry[0] is not plan:
                plan.close()
            self._close(evicted)
        plan, lock, _ = entry
        with lock:
            if plan.is_open:
                return plan.run_host(array)
        with make() as fresh:  # evicted by another thread meanwhile
            return fresh.run_host(array)

    def clear(self) -> None:
        with self._lock:
            entries = list(self._plans.values())
            self._plans.clear()
        self._close(entries)


_plan_cache = _PlanCache()


def clear_plan_cache() -> None:
    """Close every cached plan of the one-call filters."""
    _plan_cache.clear()


def _cache_key(array: np.ndarray, kind, size, footprint, origin, mode, *rest) -> tuple:
    fp = None
    if footprint is not None:
        mask = np.asarray(footprint, dtype=bool)
        fp = (mask.shape, mask.tobytes())
    return (array.shape, array.dtype.str, kind, tuple(int(v) for v in size), fp,
            None if origin is None else tuple(int(v) for v in origin),
            None if mode is None else tuple(mode), os.environ.get("NDF_MOMENTS", "fp32c"), *rest)


def _typed_array(array: object) -> np.ndarray:
    if not isinstance(array, np.ndarray) or array.dtype not in (np.float32, np.float64):
        raise TypeError("argument 'array': expected a float32 or float64 numpy.ndarray")
    return array


def window_filter(
    array,
    kind,
    size,
    footprint,
    origin,
    mode,
    cval,
    omit_nan,
    ignore_inf,
    min_count,
    parameter,
):
    """Apply one window reduction (``_core.window_filter``)."""
    array = _typed_array(array)
    if not array.flags.c_contiguous:
        raise ValueError("native input must be C-contiguous")
    cval = float(np.float32(cval)) if array.dtype == np.float32 else float(cval)

    def make() -> Plan:
        return Plan(array.shape, array.dtype, kind, size, footprint=footprint, origin=origin, mode=mode, cval=cval,
                    omit_nan=omit_nan, ignore_inf=ignore_inf, min_count=min_count, parameter=parameter)

    key = _cache_key(array, kind, size, footprint, origin, mode, np.float64(cval).tobytes(), bool(omit_nan),
                     bool(ignore_inf), int(min_count), int(parameter))
    return _plan_cache.run(key, make, array)


def robust_filter(
    array,
    size,
    footprint,
    origin,
    mode,
    cval,
    kind,
    parameter,
    omit_nan,
    ignore_inf,
    min_count,
    sigma_lower,
    sigma_upper,
    maxiters,
    center,
    spread,
    estimator="sex",
    modify_sample_size=False,
    pearson=2.5,
):
    """Apply one robust window statistic (``_core.robust_filter``,
    src/pyapi/robust.rs:78-171): the percentile, the MAD, iterative sigma
    clipping (``sigma_mean`` / ``sigma_median`` / ``sigma_mode``), the mode
    estimators and the biweight location / scale."""
    clip = kind in ("sigma_mean", "sigma_median", "sigma_mode")
    if kind not in ("percentile",) + ROBUST_KINDS:
        raise ValueError("unsupported robust filter kind")
    if not clip and not omit_nan and (ignore_inf or min_count != 1):
        raise ValueError("ignore_inf and min_count require NaN omission")
    if kind in ("mode", "sigma_mode") and estimator not in ESTIMATORS:
        raise ValueError("mode estimator must be 'sex', 'mmm', or 'iraf'")
    if clip:
        if center not in CENTERS:
            raise ValueError("center must be 'mean' or 'median'")
        if spread not in SPREADS:
            raise ValueError("spread must be 'std' or 'mad'")
    array = _typed_array(array)
    if not array.flags.c_contiguous or not array.flags.aligned:
        raise ValueError("native input must be aligned and C-contiguous")
    options = dict(parameter=parameter, sigma_lower=sigma_lower, sigma_upper=sigma_upper,
                   maxiters=maxiters, center=center if clip else "median",
                   spread=spread if clip else "std",
                   estimator=estimator if kind in ("mode", "sigma_mode") else "sex",
                   modify_sample_size=modify_sample_size, pearson=pearson)
    def make() -> Plan:
        return Plan(array.shape, array.dtype, kind, size, footprint=footprint, origin=origin, mode=mode,
                    cval=float(cval), omit_nan=True if clip else omit_nan, ignore_inf=True if clip else ignore_inf,
                    min_count=min_count, percentile=float(parameter), robust=options)

    key = _cache_key(array, kind, size, footprint, origin, mode, np.float64(cval).tobytes(), bool(omit_nan),
                     bool(ignore_inf), int(min_count), np.float64(parameter).tobytes(),
                     tuple((k, np.float64(v).tobytes() if isinstance(v, float) else v)
                           for k, v in sorted(options.items())))
    return _plan_cache.run(key, make, array)


def _unsupported(name: str) -> ValueError:
    return ValueError(f"unsupported {name}")


def mesh_config(estimator, sigma_lower, sigma_upper, maxiters, center, spread, statistic, mode_estimator,
                pearson, rms, min_valid_fraction, valid_count, valid_base, fill, idw_neighbors, idw_power,
                filter_edge, filter_threshold, threshold_kind, interpolation) -> MeshConfig:
    """The MeshConfig of src/pyapi/background.rs:42-123 (string options parsed
    in the same order, with the same messages)."""
    choices = {
        "estimator": {"sextractor": 0, "sigma_clip": 1},
        "valid_count": {"finite": 0, "retained": 1},
        "valid_base": {"mesh": 0, "box": 1},
        "fill": {"nearest": 0, "idw": 1},
        "filter_edge": {"shrink": 0, "truncate": 1},
        "interpolation": {"spline": 0, "sextractor": 1},
    }

    def pick(name, value, table):
        if value not in table:
            raise _unsupported(name)
        return table[value]

    est = pick("estimator", estimator, choices["estimator"])
    mode_code, center_code, spread_code, statistic_code, rms_code = 0, 1, 0, 2, 0
    if est == 1:
        mode_code = pick("mode_estimator", mode_estimator, ESTIMATORS)
        center_code = pick("center", center, CENTERS)
        spread_code = pick("spread", spread, SPREADS)
        statistic_code = pick("statistic", statistic, {"mean": 0, "median": 1, "mode": 2})
        rms_code = pick("rms", rms, {"std": 0, "mad": 1})
    count = pick("valid_count", valid_count, choices["valid_count"])
    base = pick("valid_base", valid_base, choices["valid_base"])
    fill_code = pick("fill", fill, choices["fill"])
    edge = pick("filter_edge", filter_edge, choices["filter_edge"])
    if threshold_kind not in ("deviation", "above"):
        raise _unsupported("threshold_kind")
    kind = 0 if filter_threshold is None else (1 if threshold_kind == "deviation" else 2)
    interp = pick("interpolation", interpolation, choices["interpolation"])
    return MeshConfig(est, float(pearson), float(sigma_lower), float(sigma_upper),
                      -1 if maxiters is None else int(maxiters), center_code, spread_code, statistic_code,
                      mode_code, rms_code, float(min_valid_fraction), count, base, fill_code, int(idw_neighbors),
                      float(idw_power), edge, kind, 0.0 if filter_threshold is None else float(filter_threshold),
                      interp)


def mesh_background(array, mask, box_size, filter_size, estimator, sigma_lower, sigma_upper, maxiters, center,
                    spread, statistic, mode_estimator, pearson, rms, min_valid_fraction, valid_count, valid_base,
                    fill, idw_neighbors, idw_power, filter_edge, filter_threshold, threshold_kind, interpolation):
    """``_core.mesh_background`` (src/pyapi/background.rs:225-280): returns
    (background, rms, mesh_background, mesh_rms, mesh_valid,
    mesh_finite_count, mesh_retained_count, global_background, global_rms)."""
    lib, _ = _load()
    config = mesh_config(estimator, sigma_lower, sigma_upper, maxiters, center, spread, statistic, mode_estimator,
                         pearson, rms, min_valid_fraction, valid_count, valid_base, fill, idw_neighbors, idw_power,
                         filter_edge, filter_threshold, threshold_kind, interpolation)
    array = _typed_array(array)
    if not array.flags.c_contiguous or not array.flags.aligned:
        raise ValueError("native input must be aligned and C-contiguous")
    shape = array.shape
    ndim = len(shape)
    boxes, filters = list(box_size), list(filter_size)
    if len(boxes) != ndim or len(filters) != ndim:
        raise ValueError("box and filter sizes need one entry per axis")
    if any(int(b) == 0 for b in boxes):
        raise ValueError("box sizes must be positive")
    mesh_shape = tuple(-(-int(n) // int(b)) for n, b in zip(shape, boxes))
    flags = None
    if mask is not None:
        flags = np.ascontiguousarray(mask, dtype=np.uint8)
        if flags.shape != shape:
            raise ValueError("mask must have the same shape as data")
    # Both maps are written whole by the device pipeline.
    background = _host_buffers.array(shape, array.dtype) if array.size else np.zeros(shape, dtype=array.dtype)
    rms_map = _host_buffers.array(shape, array.dtype) if array.size else np.zeros(shape, dtype=array.dtype)
    mesh_bg = np.zeros(mesh_shape, np.float64)
    mesh_rms = np.zeros(mesh_shape, np.float64)
    valid = np.zeros(mesh_shape, np.uint8)
    finite = np.zeros(mesh_shape, np.int64)
    retained = np.zeros(mesh_shape, np.int64)
    globals_ = np.zeros(2, np.float64)
    ptr = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
    _check(lib.ndf_mesh_background(
        array.ctypes.data_as(ctypes.c_void_p), None if flags is None else ptr(flags, ctypes.c_uint8),
        0 if array.dtype == np.float32 else 1, ndim, _u64(shape), _u64(boxes), _u64(filters),
        ctypes.byref(config), background.ctypes.data_as(ctypes.c_void_p),
        rms_map.ctypes.data_as(ctypes.c_void_p), ptr(mesh_bg, ctypes.c_double), ptr(mesh_rms, ctypes.c_double),
        ptr(valid, ctypes.c_uint8), ptr(finite, ctypes.c_int64), ptr(retained, ctypes.c_int64),
        ptr(globals_, ctypes.c_double)), lib)
    return (background, rms_map, mesh_bg, mesh_rms, valid.astype(bool), finite, retained, float(globals_[0]),
            float(globals_[1]))


def get_num_threads() -> int:
    """Number of host threads in the library's host-side pool.

    Like the reference's global Rayon pool it honours ``RAYON_NUM_THREADS``
    (a positive integer) read once per process; otherwise it is the hardware
    thread count capped at 16. The device work is spread over the GPU's SMs
    regardless (``device_info()["sm_count"]``).
    """
    lib, _ = _load()
    return int(lib.ndf_get_num_threads())


def device_info() -> dict:
    lib, _ = _load()
    sms, major, minor = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    name = ctypes.create_string_buffer(256)
    _check(
        lib.ndf_device_info(ctypes.byref(sms), ctypes.byref(major), ctypes.byref(minor), name, 256),
        lib,
    )
    return {
        "sm_count": sms.value,
        "capability": (major.value, minor.value),
        "name": name.value.decode(),
    }


def set_autotune(mode: int, cache_path: str | None = None) -> None:
    """Kernel-choice autotuner: 0 off, 1 plans use measured choices and
    batches measure what they miss (default), 2 every plan measures what it
    misses. ``cache_path``: None keeps the current file, "" keeps choices in
    memory only. Choices change speed only, never results."""
    lib, _ = _load()
    path = None if cache_path is None else str(cache_path).encode()
    _check(lib.ndf_set_autotune(int(mode), path), lib)
    _plan_cache.clear()


def autotune_entries() -> int:
    """Number of measured kernel choices known to the autotuner."""
    lib, _ = _load()
    return int(lib.ndf_autotune_entries())


def pin_kernel(family: str | None) -> None:
    """Make plans take kernel ``family`` ("histogram", "box", "network",
    "ranked", "radix", "moments", "slide", "extrema", "passes", "boxcar",
    "band")
    whenever it is one of their candidates; None unpins. Results never
    depend on it."""
    lib, _ = _load()
    _check(lib.ndf_pin_kernel(None if family is None else str(family).encode()), lib)
    _plan_cache.clear()


def set_tma(enabled: bool) -> None:
    """Turn TMA staging of interior tiles on (default) or off; results are
    identical either way."""
    lib, _ = _load()
    _check(lib.ndf_set_tma(int(bool(enabled))), lib)


def selftest_wait_timeout() -> int:
    """Run the bounded-wait self-test; returns the library status code, which
    is 7 (NDF_ERR_TIMEOUT) when the wait gave up and reported it."""
    lib, _ = _load()
    return int(lib.ndf_selftest_wait_timeout())
