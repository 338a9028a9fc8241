"""Generate the committed mesh-background golden vectors (``mesh_v1.npz``).

The expected outputs come from the reference project's own independent NumPy
statement of the pipeline, ``tests/_background_reference.py``
(``mesh_background``), imported from a checkout of ysBach/ndfiltrs v0.2.0,
over the case matrix of its ``tests/test_background.py``
(``test_matches_numpy_reference``): sloped Gaussian noise with bright sources
and NaNs, a masked corner, SExtractor and photutils rule sets, 1-D / 2-D / 3-D
shapes, partial edge meshes, filter thresholds. The reference compares its
native pipeline with this statement within 1e-11 absolute (Neumaier against
pairwise sums, and a different tridiagonal solver); the oracle is pinned the
same way.

Run (needs the reference checkout and SciPy; not needed to use the fixture):

    python tests/golden/make_mesh_golden.py --reference /path/to/ndfiltrs
"""

from __future__ import annotations

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

PHOTUTILS = {
    "estimator": "sigma_clip",
    "maxiters": 10,
    "statistic": "mode",
    "mode_estimator": "sex",
    "rms": "std",
    "min_valid_fraction": 0.9,
    "valid_count": "retained",
    "valid_base": "box",
    "fill": "idw",
    "filter_edge": "truncate",
}

CASES = [
    ((150, 230), (32, 40), {}),
    ((150, 230), (32, 40), {"mode_estimator": "mmm"}),
    ((150, 230), (25, 25), PHOTUTILS),
    ((120, 90), (16, 30), {"filter_size": (3, 5), "filter_threshold": 0.5}),
    ((120, 90), (16, 30), {**PHOTUTILS, "filter_threshold": 101.0, "threshold_kind": "above"}),
    ((97,), (10,), {"filter_size": 5}),
    ((20, 18, 15), (6, 5, 4), {}),
    ((20, 18, 15), (6, 5, 4), {**PHOTUTILS, "spread": "mad", "rms": "mad"}),
    ((64, 64), (64, 64), {}),
]

SAMPLE = 11
FIELDS = ("background", "rms", "mesh_background", "mesh_rms", "mesh_valid", "mesh_finite_count",
          "mesh_retained_count", "global_background", "global_rms")


def image(shape: tuple[int, ...], seed: int) -> np.ndarray:
    """Sloped Gaussian noise (sigma 5) with bright sources and NaNs."""
    rng = np.random.default_rng(seed)
    grids = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    values = 100.0 + sum(0.02 * (axis + 1) * g for axis, g in enumerate(grids))
    values = values + rng.normal(0.0, 5.0, shape)
    flat = values.reshape(-1)
    flat[rng.choice(flat.size, flat.size // 200, replace=False)] += 800.0
    flat[rng.choice(flat.size, flat.size // 300, replace=False)] = np.nan
    return values


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument(
        "--reference",
        default=os.environ.get("NDFILTRS_REFERENCE"),
        help="checkout of the reference project (or set NDFILTRS_REFERENCE)",
    )
    parser.add_argument("--output", default=str(HERE / "mesh_v1"))
    args = parser.parse_args()
    if not args.reference:
        parser.error("--reference (or NDFILTRS_REFERENCE) is required")
    sys.path.insert(0, args.reference)
    from tests._background_reference import mesh_background as reference

    arrays: dict[str, np.ndarray] = {}
    cases = []
    for index, (shape, box, options) in enumerate(CASES):
        data = image(shape, seed=len(shape) + sum(box))
        mask = np.zeros(shape, dtype=bool)
        mask[tuple(slice(0, n // 3) for n in shape)] = True
        expected = reference(data, box, mask=mask, **options)
        # Inputs are regenerated from the seed by the tests; the
        # full-resolution maps are kept at every 11th pixel (C order).
        for name in FIELDS:
            value = np.asarray(expected[name])
            if name in ("background", "rms"):
                value = value.reshape(-1)[::SAMPLE]
            arrays[f"{name}{index}"] = value
        cases.append({"index": index, "shape": list(shape), "box": list(box),
                      "options": {k: list(v) if isinstance(v, tuple) else v for k, v in options.items()}})
    np.savez_compressed(args.output + ".npz", **arrays)
    Path(args.output + ".json").write_text(json.dumps(cases, indent=1))
    print(f"{len(cases)} cases -> {args.output}.npz")


if __name__ == "__main__":
    main()
