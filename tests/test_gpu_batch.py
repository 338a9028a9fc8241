"""Batched persistent path: one persistent launch per kernel family,
replayed from a CUDA graph, equals per-image plans and the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits

pytestmark = pytest.mark.gpu


def _specs(rng, count):
    from ndfiltrs_gb300 import kernels

    specs, images = [], []
    for i in range(count):
        h = int(np.exp(rng.uniform(np.log(40), np.log(300))))
        w = int(np.exp(rng.uniform(np.log(40), np.log(300))))
        image = rng.normal(1000, 10, size=(h, w)).astype(np.float32)
        image[rng.random(image.shape) < 0.01] = np.nan
        image[rng.random(image.shape) < 0.002] = rng.uniform(2000, 60000)
        window = int(rng.choice([3, 5, 7, 9, 11, 13, 15]))
        shape_kind = ["box", "tophat", "ring"][i % 3]
        footprint = None
        size = (window, window)
        if shape_kind == "tophat":
            footprint = kernels.tophat(window // 2, 2) != 0
        elif shape_kind == "ring":
            outer = max(window // 2, 2)
            footprint = kernels.ring(outer - 2, outer, 2) != 0
        kind = ["median", "percentile", "std"][(i // 3) % 3]
        spec = dict(shape=image.shape, kind=kind, size=size, footprint=footprint, omit_nan=True,
                    ignore_inf=kind == "std", min_count=1, parameter=1 if kind == "std" else 0,
                    percentile=84.0, mode=["reflect", "nearest", "mirror", "wrap", "constant"][i % 5])
        specs.append(spec)
        images.append(image)
    return specs, images


def test_batch_matches_per_image_plans_and_oracle(gpu, oracle) -> None:
    import torch

    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(5)
    specs, images = _specs(rng, 36)
    batch = _core.Batch(specs)
    device = torch.device("cuda")
    d_in = [torch.from_numpy(im).to(device) for im in images]
    d_out = [torch.full_like(t, 7.0) for t in d_in]
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # the second run replays the captured graph
        batch.run_device([t.data_ptr() for t in d_in], [t.data_ptr() for t in d_out], stream)
    torch.cuda.synchronize()
    assert 1 <= batch.launches <= len(specs)
    for spec, image, out in zip(specs, images, d_out):
        got = out.cpu().numpy()
        kw = {k: spec[k] for k in ("size", "footprint", "omit_nan", "ignore_inf", "min_count",
                                    "parameter", "percentile")}
        if spec["footprint"] is not None:
            kw["size"] = spec["footprint"].shape
        plan = _core.Plan(image.shape, np.float32, spec["kind"], mode=[spec["mode"]] * 2, **kw)
        want = plan.run_host(image)
        plan.close()
        np.testing.assert_array_equal(bits(got), bits(want), err_msg=str(spec["kind"]))
        if spec["kind"] != "std":
            ref = oracle.window_filter(image, spec["kind"], spec["size"], footprint=spec["footprint"],
                                       mode=spec["mode"], omit_nan=True, q=84.0)
            np.testing.assert_array_equal(bits(got), bits(ref))
    batch.close()


def test_batch_host_pipeline_matches_device_run(gpu) -> None:
    """ndf_batch_run_host (pageable inputs, grouped uploads, kernels and
    downloads overlapping) equals the device-buffer run, twice in a row,
    with empty images, box / histogram images (own launches) and family
    images mixed; the second call reuses the pipeline's buffers."""
    import torch

    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(11)
    specs, images = _specs(rng, 27)
    # Large windows (histogram kernel) and an empty image in the mix.
    big = rng.normal(500, 5, size=(211, 190)).astype(np.float32)
    specs.append(dict(shape=big.shape, kind="median", size=(31, 31), footprint=None, omit_nan=True,
                      ignore_inf=False, min_count=1, parameter=0, percentile=50.0, mode="nearest"))
    images.append(big)
    specs.insert(5, dict(shape=(0, 7), kind="median", size=(3, 3), footprint=None, omit_nan=True,
                         ignore_inf=False, min_count=1, parameter=0, percentile=50.0, mode="reflect"))
    images.insert(5, np.empty((0, 7), np.float32))
    batch = _core.Batch(specs)
    device = torch.device("cuda")
    d_in = [torch.from_numpy(im).to(device) for im in images]
    d_out = [torch.empty_like(t) for t in d_in]
    stream = torch.cuda.current_stream().cuda_stream
    batch.run_device([t.data_ptr() for t in d_in], [t.data_ptr() for t in d_out], stream)
    torch.cuda.synchronize()
    expected = [t.cpu().numpy() for t in d_out]
    for _ in range(2):
        got = batch.run_host(images)
        for want, have, spec in zip(expected, got, specs):
            assert have.shape == want.shape
            np.testing.assert_array_equal(bits(have), bits(want), err_msg=str(spec["kind"]))
    outputs = [np.full(im.shape, 3.0, np.float32) for im in images]
    assert batch.run_host(images, outputs) is outputs
    for want, have in zip(expected, outputs):
        np.testing.assert_array_equal(bits(have), bits(want))
    batch.close()


def test_batch_with_rolling_means_extrema_and_robust_kinds(gpu) -> None:
    """Images whose plans use the band rolling mean, the two-pass extrema or
    the robust kernel run their own launches inside the batch's graph; the
    results equal per-image plans, on device buffers and through the host
    pipeline."""
    import torch

    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(17)
    kinds = [("mean_rolling", (31, 31), {}), ("min", (9, 9), {}), ("max", (1, 15), {}),
             ("mad", (5, 5), {"parameter": 1.4826}),
             ("sigma_median", (7, 7), {"sigma_lower": 2.0, "sigma_upper": 2.0, "maxiters": None}),
             ("biweight_location", (5, 5), {"parameter": 6.0}), ("median", (5, 5), {})]
    specs, images = [], []
    for i in range(21):
        kind, size, robust = kinds[i % len(kinds)]
        image = rng.normal(1000, 10, size=(int(rng.integers(30, 200)), int(rng.integers(30, 200))))
        image = image.astype(np.float32)
        image[rng.random(image.shape) < 0.02] = np.nan
        specs.append(dict(shape=image.shape, kind=kind, size=size, footprint=None, omit_nan=True,
                          ignore_inf=False, min_count=1, parameter=0, percentile=50.0,
                          mode=["reflect", "nearest", "wrap"][i % 3], robust=robust))
        images.append(image)
    batch = _core.Batch(specs)
    device = torch.device("cuda")
    d_in = [torch.from_numpy(im).to(device) for im in images]
    d_out = [torch.full_like(t, 7.0) for t in d_in]
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        batch.run_device([t.data_ptr() for t in d_in], [t.data_ptr() for t in d_out], stream)
    torch.cuda.synchronize()
    hosted = batch.run_host(images)
    for spec, image, out, host in zip(specs, images, d_out, hosted):
        with _core.Plan(image.shape, np.float32, spec["kind"], spec["size"], mode=[spec["mode"]] * 2,
                        omit_nan=True, robust=spec["robust"]) as plan:
            want = plan.run_host(image)
        np.testing.assert_array_equal(bits(out.cpu().numpy()), bits(want), err_msg=spec["kind"])
        np.testing.assert_array_equal(bits(host), bits(want), err_msg=spec["kind"])
    batch.close()


def test_specialised_kernels_run_as_one_persistent_launch_per_family(gpu) -> None:
    """Images whose plans take the box-pair kernel, the sliding histogram,
    the sliding exact moments or the ranked network join one persistent
    launch per family (kernel and variant) instead of launching per image;
    results equal per-image plans bit for bit."""
    import torch

    from ndfiltrs_gb300 import _core

    rng = np.random.default_rng(11)
    specs, images = [], []
    families = [("median", (5, 5), "tile_box"), ("median_histogram", (33, 31), "histogram"),
                ("std", (9, 9), "moments_slide"), ("median", (9, 9), "rank_network")]
    for i in range(16):
        kind, size, _ = families[i % 4]
        image = rng.normal(1000, 10, size=(int(rng.integers(60, 260)), int(rng.integers(60, 260))))
        image = image.astype(np.float32)
        image[rng.random(image.shape) < 0.02] = np.nan
        specs.append(dict(shape=image.shape, kind=kind, size=size, footprint=None, omit_nan=True,
                          ignore_inf=kind == "std", min_count=1, parameter=1 if kind == "std" else 0,
                          percentile=50.0, mode=["reflect", "nearest", "wrap"][i % 3]))
        images.append(image)
    wants = []
    for i, (spec, image) in enumerate(zip(specs, images)):
        with _core.Plan(image.shape, np.float32, spec["kind"], spec["size"], mode=[spec["mode"]] * 2,
                        omit_nan=True, ignore_inf=spec["ignore_inf"], parameter=spec["parameter"]) as plan:
            assert plan.algorithm == families[i % 4][2], (spec["kind"], spec["size"], plan.algorithm)
            wants.append(plan.run_host(image))
    batch = _core.Batch(specs)
    d_in = [torch.from_numpy(im).cuda() for im in images]
    d_out = [torch.full_like(t, 3.0) for t in d_in]
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        batch.run_device([t.data_ptr() for t in d_in], [t.data_ptr() for t in d_out], stream)
    torch.cuda.synchronize()
    assert batch.launches == 4
    for spec, out, want in zip(specs, d_out, wants):
        np.testing.assert_array_equal(bits(out.cpu().numpy()), bits(want), err_msg=spec["kind"])
    hosts = batch.run_host(images)
    for spec, host, want in zip(specs, hosts, wants):
        np.testing.assert_array_equal(bits(host), bits(want), err_msg=spec["kind"])
