"""The allocation-free histogram entry point (``ndf_histogram_filter_noalloc``).

It exists for callers that cannot let a library allocate device memory
(code running during stream capture, frameworks that own all device memory,
real-time pipelines that cannot absorb an allocation's implicit device
synchronization). Its sort scratch lives in a static device array of the
library instead of a cudaMalloc'd workspace. This test calls it through the
C-ABI on caller-owned device buffers and checks two calls in a row against
the regular plan entry point (``ndf_plan_*``); order statistics must match
bit for bit. The file is named to be collected last.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = {"median": 0, "median_histogram": 2, "rank": 9}
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
    image[:, shape[1] // 3] = np.nan
    return image


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_no_alloc_entry_point_matches_plan_entry_point(gpu, dtype) -> None:
    import torch

    from ndfiltrs_gb300 import _core

    lib, fn = _entry_point()
    cases = [
        (_image((300, 280), dtype, 1), "median_histogram", (33, 31), (0, 0), ("nearest", "nearest"),
         True, False, 1, 0),
        (_image((257, 190), dtype, 2), "rank", (9, 12), (1, -3), ("wrap", "reflect"),
         False, False, 1, 20),
    ]
    stream = torch.cuda.current_stream().cuda_stream
    for image, kind, size, origin, mode, omit, ignore_inf, min_count, parameter in cases:
        with _core.Plan(image.shape, dtype, kind, size, origin=origin, mode=mode, cval=0.0,
                        omit_nan=omit, ignore_inf=ignore_inf, min_count=min_count,
                        parameter=parameter) as plan:
            expected = plan.run_host(image)
        d_in = torch.from_numpy(image).cuda()
        d_out = torch.full_like(d_in, 123.0)
        u64 = ctypes.c_uint64 * 2
        rc = fn(
            d_in.data_ptr(), d_out.data_ptr(), 0 if dtype == np.float32 else 1, 2,
            u64(*image.shape), u64(*size), (ctypes.c_int64 * 2)(*origin),
            (ctypes.c_int32 * 2)(*[MODES[m] for m in mode]), 0.0, KINDS[kind], int(omit),
            int(ignore_inf), min_count, parameter, 50.0, stream,
        )
        assert rc == 0, lib.ndf_last_error().decode()
        torch.cuda.synchronize()
        actual = d_out.cpu().numpy()
        bits = np.uint32 if dtype == np.float32 else np.uint64
        np.testing.assert_array_equal(actual.view(bits), expected.view(bits), err_msg=kind)
