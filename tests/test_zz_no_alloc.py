"""The allocation-free histogram entry point (``ndf_histogram_filter_noalloc``).

It exists for callers that cannot let a library allocate device memory:
code that runs while a CUDA stream is being captured (cudaMalloc is not
allowed there), frameworks that own all device memory through their own
pool, and real-time pipelines that cannot absorb an allocation's implicit
device synchronization. Its sort scratch lives in a static device array of
the library instead of a cudaMalloc'd workspace.

These tests call it through the C-ABI on caller-owned device buffers:

* two calls in a row against the regular plan entry point (``ndf_plan_*``),
  bit for bit;
* every statistic it offers (median, rank, min, max, and percentiles whose
  rank split is computed on the device) on 1-D and 2-D arrays, both dtypes,
  both NaN policies (with ``ignore_inf`` and ``min_count``), every boundary
  mode (constant with a non-zero ``cval``), against the CPU oracle bit for
  bit;
* after a warm-up pass, a second pass over every case leaves the device's
  free memory unchanged (no allocation, no free).

The file is named to be collected last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = {"median": 0, "median_histogram": 2, "min": 5, "max": 6, "rank": 9, "rank_histogram": 10,
         "percentile": 11}
MODES = {"reflect": 0, "constant": 1, "nearest": 2, "mirror": 3, "wrap": 4}


def _entry_point():
    from ndfiltrs_gb300 import _core

    lib, _ = _core._load()
    fn = lib.ndf_histogram_filter_noalloc
    fn.argtypes = [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
        ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
        ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32), ctypes.c_double,
        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64,
        ctypes.c_double, ctypes.c_void_p,
    ]
    fn.restype = ctypes.c_int
    return lib, fn


def _image(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    image = (500 + rng.normal(size=shape) * 20).astype(dtype)
    image[rng.random(shape) < 0.02] = np.nan
    image[rng.random(shape) < 0.005] = np.inf
    image[rng.random(shape) < 0.005] = -np.inf
    image.flat[::97] = -0.0
    if image.ndim == 2:
        image[:, shape[1] // 3] = np.nan
    return image


def _bits(array: np.ndarray) -> np.ndarray:
    return array.view(np.uint32 if array.dtype == np.float32 else np.uint64)


def _call(fn, lib, d_in, d_out, dtype, shape, case, stream) -> None:
    ndim = len(shape)
    rc = fn(
        d_in.data_ptr(), d_out.data_ptr(), 0 if dtype == np.float32 else 1, ndim,
        (ctypes.c_uint64 * ndim)(*shape), (ctypes.c_uint64 * ndim)(*case["size"]),
        (ctypes.c_int64 * ndim)(*case["origin"]),
        (ctypes.c_int32 * ndim)(*[MODES[m] for m in case["mode"]]), case["cval"],
        KINDS[case["kind"]], int(case["omit"]), int(case["ignore_inf"]), case["min_count"],
        case["parameter"], case["q"], stream,
    )
    assert rc == 0, lib.ndf_last_error().decode()


def _case(kind, size, origin, mode, *, omit=True, ignore_inf=False, min_count=1, parameter=0, q=50.0,
          cval=0.0):
    return dict(kind=kind, size=size, origin=origin, mode=mode, omit=omit, ignore_inf=ignore_inf,
                min_count=min_count, parameter=parameter, q=q, cval=cval)


def _oracle_cases():
    """(shape, case) pairs over every statistic, policy, mode and rank."""
    two = (211, 173)
    one = (4099,)
    return [
        (two, _case("median_histogram", (33, 31), (0, 0), ("nearest", "nearest"))),
        (two, _case("median", (21, 24), (-3, 5), ("reflect", "mirror"), omit=False)),
        (two, _case("rank_histogram", (17, 19), (2, -4), ("wrap", "constant"), omit=False, parameter=37,
                    cval=-7.25)),
        (two, _case("min", (25, 25), (0, 0), ("constant", "constant"), cval=3.5, ignore_inf=True)),
        (two, _case("max", (19, 41), (1, -2), ("mirror", "nearest"), min_count=200)),
        (two, _case("percentile", (29, 27), (0, 1), ("reflect", "wrap"), q=16.0)),
        (two, _case("percentile", (29, 27), (-2, 0), ("nearest", "constant"), q=84.0, cval=601.0,
                    ignore_inf=True, min_count=300)),
        (two, _case("percentile", (15, 35), (0, 0), ("reflect", "reflect"), omit=False, q=84.0)),
        (one, _case("median_histogram", (101,), (0,), ("reflect",))),
        (one, _case("percentile", (64,), (-7,), ("constant",), q=16.0, cval=-1.5, ignore_inf=True,
                    min_count=20)),
        (one, _case("max", (257,), (100,), ("wrap",), omit=False)),
        (one, _case("rank", (40,), (3,), ("mirror",), parameter=11)),
    ]


def _oracle(oracle, image, case):
    kind = case["kind"]
    return oracle.window_filter(
        image, kind, case["size"], origin=case["origin"], mode=case["mode"], cval=case["cval"],
        omit_nan=case["omit"], ignore_inf=case["ignore_inf"], min_count=case["min_count"],
        parameter=case["parameter"], q=case["q"], direct=True,
    )


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_no_alloc_entry_point_matches_plan_entry_point(gpu, dtype) -> None:
    """Two calls in a row each equal the plan entry point's result."""
    import torch

    from ndfiltrs_gb300 import _core

    lib, fn = _entry_point()
    cases = [
        ((300, 280), 1, _case("median_histogram", (33, 31), (0, 0), ("nearest", "nearest"))),
        ((257, 190), 2, _case("rank", (9, 12), (1, -3), ("wrap", "reflect"), omit=False, parameter=20)),
    ]
    stream = torch.cuda.current_stream().cuda_stream
    for shape, seed, case in cases:
        image = _image(shape, dtype, seed)
        with _core.Plan(image.shape, dtype, case["kind"], case["size"], origin=case["origin"],
                        mode=case["mode"], cval=0.0, omit_nan=case["omit"],
                        ignore_inf=case["ignore_inf"], min_count=case["min_count"],
                        parameter=case["parameter"]) as plan:
            expected = plan.run_host(image)
        d_in = torch.from_numpy(image).cuda()
        for _ in range(2):
            d_out = torch.full_like(d_in, 123.0)
            _call(fn, lib, d_in, d_out, dtype, shape, case, stream)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(_bits(d_out.cpu().numpy()), _bits(expected),
                                          err_msg=case["kind"])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_no_alloc_entry_point_matches_oracle_and_allocates_nothing(gpu, oracle, dtype) -> None:
    """Every statistic, policy, mode and rank against the oracle; the second
    pass over all cases leaves the device's free memory where it was."""
    import torch

    lib, fn = _entry_point()
    stream = torch.cuda.current_stream().cuda_stream
    work = []
    for seed, (shape, case) in enumerate(_oracle_cases()):
        image = _image(shape, dtype, 10 + seed)
        expected = _oracle(oracle, image, case)
        d_in = torch.from_numpy(image).cuda()
        d_out = torch.empty_like(d_in)
        work.append((shape, case, expected, d_in, d_out))
    torch.cuda.synchronize()
    free_before = None
    for attempt in range(2):
        for shape, case, expected, d_in, d_out in work:
            d_out.fill_(123.0)
        torch.cuda.synchronize()
        if attempt == 1:
            free_before = torch.cuda.mem_get_info()[0]
        for shape, case, expected, d_in, d_out in work:
            _call(fn, lib, d_in, d_out, dtype, shape, case, stream)
        torch.cuda.synchronize()
        if attempt == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        for shape, case, expected, d_in, d_out in work:
            label = f"{case['kind']} {shape} {case}"
            np.testing.assert_array_equal(_bits(d_out.cpu().numpy()), _bits(expected), err_msg=label)


def test_no_alloc_entry_point_rejects_what_it_cannot_do(gpu) -> None:
    """Sizes beyond its limits and non-order statistics come back as errors."""
    import torch

    lib, fn = _entry_point()
    stream = torch.cuda.current_stream().cuda_stream
    d = torch.zeros(64, dtype=torch.float32, device="cuda")
    u64 = ctypes.c_uint64

    def status(shape, size, kind=0):
        n = len(shape)
        return fn(d.data_ptr(), d.data_ptr(), 0, n, (u64 * n)(*shape), (u64 * n)(*size),
                  (ctypes.c_int64 * n)(*([0] * n)), (ctypes.c_int32 * n)(*([0] * n)), 0.0, kind, 1, 0, 1, 0,
                  50.0, stream)

    assert status((8, 8), (3, 3), kind=3) == 8  # mean: out of scope for this entry point
    assert status((4, 4, 4), (3, 3, 3)) == 8  # 3-D arrays
    assert status((1 << 40, 1 << 40), (3, 3)) == 5  # shape product overflows
    assert status((8,), (70000,)) == 5  # window beyond the rank-code range
