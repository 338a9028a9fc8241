"""The pool of host output buffers (``_core._HostBuffers``): outputs are
writable C-contiguous arrays of the requested shape and dtype, a buffer is
reused only after every array viewing it is released, and idle buffers stay
within their cap."""

from __future__ import annotations

import gc

import numpy as np

from ndfiltrs_gb300 import _core


def test_reuse_only_after_release() -> None:
    pool = _core._HostBuffers(max_idle_bytes=16 << 20)
    a = pool.array((1024, 1024), np.float32)
    assert a.shape == (1024, 1024) and a.dtype == np.float32
    assert a.flags.writeable and a.flags.c_contiguous
    first = a.ctypes.data
    b = pool.array((1024, 1024), np.float32)
    assert b.ctypes.data != first
    view = a[5:]
    del a
    gc.collect()
    c = pool.array((1024, 1024), np.float32)
    assert c.ctypes.data not in (first, b.ctypes.data)  # `view` still holds the first buffer
    del view
    gc.collect()
    d = pool.array((1024, 1024), np.float32)
    assert d.ctypes.data == first
    d[:] = 1.5
    assert float(d.sum()) == 1.5 * d.size


def test_small_arrays_and_cap() -> None:
    pool = _core._HostBuffers(max_idle_bytes=8 << 20)
    small = pool.array((10, 10), np.float64)
    assert small.base is None and not small.any()
    arrays = [pool.array((1 << 20,), np.float32) for _ in range(4)]  # 4 MiB each
    del arrays
    gc.collect()
    assert pool._idle <= 8 << 20
