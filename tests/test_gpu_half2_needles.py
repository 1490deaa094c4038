"""The half2 raster on its hardest inputs: long, thin, tilted splats.

The half2 form evaluates each pixel's exponent in f16 from the splat's
Cholesky factor about the warp patch centre (raster_half2.cuh). The
screen-space low-pass filter (filterVariance, ProjectionStage.ts) bounds the
factor; without it a splat may be far thinner than a pixel, past f16's
resolution, and the pass renders such launches with the FP32 evaluation. Both
sides stay within the fast forms' stated tolerance of the FP32 oracle
(max abs 2e-2) and at least 50 dB against the FP64 oracle.
"""
import importlib

import numpy as np
import pytest

import oracle
from conftest import PKG_NAME
from gpu_harness import GpuRun, psnr

pytestmark = pytest.mark.gpu

sc = importlib.import_module(PKG_NAME + ".scenes")


def needle_cloud(n: int, seed: int, aspect=(30.0, 200.0), opacity_logit=(3.0, 2.0)) -> dict:
    """Splats with one long axis (ln-scale N(-1.5, 0.8)) and two axes shorter
    by a factor of 30-200, uniform rotations, opacities up to ~1 (the 0.99
    alpha clamp is active for many)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    means = rng.uniform(-3.0, 3.0, (n, 3)).astype(np.float32)
    long_axis = rng.normal(-1.5, 0.8, n)
    thin = long_axis - np.log(rng.uniform(aspect[0], aspect[1], n))
    ls = np.stack([long_axis, thin, thin + rng.normal(0.0, 0.3, n)], 1).astype(np.float32)
    op = (1.0 / (1.0 + np.exp(-rng.normal(opacity_logit[0], opacity_logit[1], n)))).astype(np.float32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 3] < 0] *= -1
    sh = np.zeros((n, 16, 3), np.float32)
    sh[:, 0, :] = (rng.uniform(0, 1, (n, 3)) - 0.5) / sc.SH_C0
    sh[:, 1:, :] = rng.normal(0, 0.1, (n, 15, 3))
    return sc.pack_scene(means, np.zeros(n), ls, op, q.astype(np.float32), sh)


@pytest.mark.parametrize("filter_variance", [0.3, 0.05, 0.01, 0.0])
def test_half2_needles_within_tolerance(filter_variance):
    scene = needle_cloud(6000, seed=91)
    frame = sc.make_frame(sc.look_at((0.5, 1.0, 9.0), (0, 0, 0)), 240, 160, 55.0, 0.1, 100.0,
                          filter_variance=filter_variance)
    o = oracle.render(scene, frame, 0)
    o64 = oracle.render(scene, frame, 1)
    run = GpuRun(scene, frame, "half2", capacity=max(int(o["state"][1]), 1))
    g = run.render(frame)
    run.close()
    assert np.array_equal(g["tile_counts"], o["tile_counts"])  # the integer stages stay exact
    err = np.abs(g["rgba"] - o["rgba"]).max()
    assert err <= 2e-2, err
    assert psnr(g["rgba"][..., :3], o64["rgba"][..., :3]) >= 50.0
