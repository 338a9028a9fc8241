"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/ndfiltrs_gb300.h. No compute call is made (no GPU)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "ndfiltrs_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ndf_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_reference_facing_entry_points() -> None:
    names = declared_functions()
    for required in ("ndf_window_filter", "ndf_robust_filter", "ndf_get_num_threads",
                     "ndf_plan_create", "ndf_plan_run", "ndf_plan_run_host"):
        assert required in names


def test_library_loads_and_exports_every_declared_symbol() -> None:
    from ndfiltrs_gb300 import _build

    path = _build.build()
    library = ctypes.CDLL(str(path))
    missing = [name for name in declared_functions() if not hasattr(library, name)]
    assert not missing, missing


def test_library_targets_sm103a_only() -> None:
    from ndfiltrs_gb300 import _build

    assert _build.ARCH == "-gencode=arch=compute_103a,code=sm_103a"
    assert "-fmad=false" not in _build.NVCC_FLAGS


def test_errors_are_values_without_a_device() -> None:
    """Validation errors come back as status codes with a message."""
    from ndfiltrs_gb300 import _core

    lib, _ = _core._load()
    handle = ctypes.c_void_p()
    shape = (ctypes.c_uint64 * 1)(4)
    size = (ctypes.c_uint64 * 1)(3)
    origin = (ctypes.c_int64 * 1)(2)  # outside -(3 // 2) ..= (3 - 1) // 2
    modes = (ctypes.c_int32 * 1)(0)
    desc = _core.FilterDesc(0, 1, shape, size, None, origin, modes, 0.0, 0, 0, 0, 1, 0, 50.0, 0)
    code = lib.ndf_plan_create(ctypes.byref(desc), ctypes.byref(handle))
    assert code == 2
    assert b"origin must satisfy" in lib.ndf_last_error()


def test_no_cpu_fallback_without_device(monkeypatch) -> None:
    """Without a CUDA device a compute call raises instead of computing on the host."""
    import numpy as np

    import ndfiltrs_gb300 as nf

    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present")
    except ImportError:
        pass
    with pytest.raises(RuntimeError, match="CUDA device"):
        nf.median_filter(np.ones((4, 4), dtype=np.float32), 3)


@pytest.mark.parametrize("threads", [1, 2, 4])
def test_fresh_process_observes_rayon_thread_count(threads: int) -> None:
    """get_num_threads needs no device and honours RAYON_NUM_THREADS like the
    reference's pool (tests/test_parallel.py:9-21 of the reference)."""
    import os
    import subprocess
    import sys

    env = dict(os.environ, RAYON_NUM_THREADS=str(threads))
    result = subprocess.run(
        [sys.executable, "-c", "import ndfiltrs_gb300 as nf; print(nf.get_num_threads())"],
        check=True, capture_output=True, text=True, env=env, cwd=str(ROOT),
    )
    assert result.stdout.strip() == str(threads)
