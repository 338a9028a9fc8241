"""Build recipe of the CUDA library ``libndfiltrs_gb300.so`` (sm_103a only).

Each ``csrc/*.cu`` translation unit compiles in parallel with nvcc; the
objects link into one shared library inside the package (in-tree, so the
loaded ``.so`` is visibly this project's). A stamp of the sources and flags
skips rebuilding when nothing changed.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
SOURCES = PACKAGE / "csrc"
INCLUDE = PACKAGE.parent / "include"
BUILD = PACKAGE / "_build"
LIBRARY = BUILD / "libndfiltrs_gb300.so"
STAMP = BUILD / "stamp.txt"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    "-std=c++17",
    "-O3",
    ARCH,
    "-lineinfo",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr",
    "-extended-lambda",
]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def _fingerprint(units: list[Path]) -> str:
    digest = hashlib.sha256()
    digest.update(" ".join(NVCC_FLAGS).encode())
    headers = sorted(SOURCES.glob("*.cuh")) + sorted(SOURCES.glob("*.h"))
    headers += sorted(INCLUDE.glob("*.h"))
    for path in units + headers:
        digest.update(path.name.encode())
        digest.update(path.read_bytes())
    return digest.hexdigest()


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    """Compile and link the library; return its path."""
    units = sorted(SOURCES.glob("*.cu"))
    fingerprint = _fingerprint(units)
    if (
        not force
        and LIBRARY.exists()
        and STAMP.exists()
        and STAMP.read_text().strip() == fingerprint
    ):
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    compiler = nvcc()
    objects = [BUILD / (unit.stem + ".o") for unit in units]

    def compile_one(pair: tuple[Path, Path]) -> None:
        unit, obj = pair
        command = [compiler, *NVCC_FLAGS, "-c", str(unit), "-o", str(obj)]
        result = subprocess.run(command, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit.name}:\n{result.stderr}")
        if verbose and result.stderr:
            print(result.stderr)

    workers = jobs or max(1, min(len(units), os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=workers) as pool:
        list(pool.map(compile_one, zip(units, objects)))
    tmp = LIBRARY.with_suffix(f".so.{os.getpid()}.tmp")
    link = [compiler, "-shared", ARCH, "-o", str(tmp), *map(str, objects), "-lpthread"]
    result = subprocess.run(link, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    STAMP.write_text(fingerprint + "\n")
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose=True))
