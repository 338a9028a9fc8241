"""Shared pytest configuration.

``-m gpu`` tests call the CUDA library through its C-ABI (via the package's
ctypes binding) and compare with the CPU oracle and the golden fixtures.
``-m "not gpu"`` tests check the oracle against the reference's known answers
and golden vectors, the host-side logic, and that the C-ABI library loads and
exports every declared symbol, without touching a GPU.
"""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"

# Kernel choices stay on the built-in preference order unless a test turns
# the autotuner on, so that assertions on a plan's algorithm do not depend on
# a choice cache left by an earlier process.
os.environ.setdefault("NDF_AUTOTUNE", "0")
os.environ.setdefault("NDF_AUTOTUNE_CACHE", "")


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as module

    module.build()
    return module


@pytest.fixture(scope="session")
def golden_cases():
    meta = json.loads((GOLDEN / "golden_v1.json").read_text())
    with np.load(GOLDEN / "golden_v1.npz", allow_pickle=False) as archive:
        arrays = {name: archive[name] for name in archive.files}
    return meta["cases"], arrays


def bits(array: np.ndarray) -> np.ndarray:
    return array.view(np.uint32 if array.dtype == np.float32 else np.uint64)


@pytest.fixture(scope="session")
def gpu():
    """The package with its CUDA library loaded and a device present."""
    import ndfiltrs_gb300 as nf
    from ndfiltrs_gb300 import _build

    _build.build()
    info = nf.device_info()
    assert info["sm_count"] > 0
    return nf
