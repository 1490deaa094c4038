"""A CPU model of the half2 raster's f16 arithmetic (no GPU).

The half2 form (3dgs_tile_webgpu_gb300/csrc/raster_half2.cuh) evaluates a
pixel's exponent p' = log2(opacity) - w1^2 - w2^2 in f16, with w = L^T d from
the Cholesky factor L of the splat's conic (scaled by log2(e)/2), expanded
about the centre of the warp's 8x8 patch: the factor, w at the centre and
log2(opacity) are rounded to f16 once per record, then five fused multiply-adds
per pixel pair, each rounded to f16. This model repeats those roundings in
numpy (a fused multiply-add is formed in float64, exact for f16 operands, and
rounded once) and compares the resulting alpha with the exact one over seeded
random conics: sigma 0.001-300 px, anisotropy up to 200, any rotation, centres
around the patch. With the screen-space filter variance at or above 0.05 (the
kernel's floor for this form) the alpha error stays within 0.006, well inside
the fast forms' 2e-2 image tolerance.
"""
import numpy as np
import pytest

LOG2E = 1.0 / np.log(2.0)
F16 = np.float16


def fma16(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F16)


def model_alpha_error(n: int, filter_variance: float, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    s1 = np.exp(rng.uniform(np.log(0.001), np.log(300.0), n))
    s2 = s1 / np.exp(rng.uniform(0.0, np.log(200.0), n))
    th = rng.uniform(0.0, np.pi, n)
    c, s = np.cos(th), np.sin(th)
    # 2D covariance R diag(s1^2, s2^2) R^T plus the low-pass filter.
    cxx = c * c * s1 * s1 + s * s * s2 * s2 + filter_variance
    cxy = c * s * (s1 * s1 - s2 * s2)
    cyy = s * s * s1 * s1 + c * c * s2 * s2 + filter_variance
    det = cxx * cyy - cxy * cxy
    a, b, cc = cyy / det, -cxy / det, cxx / det  # conic
    opacity = rng.uniform(0.05, 1.0, n)
    reach = 3.0 * np.sqrt(np.maximum(s1 * s1, 0.3)) + 4.0
    cx = rng.uniform(-1.0, 1.0, n) * reach
    cy = rng.uniform(-1.0, 1.0, n) * reach
    # Staging (FP32): M = [[a, b], [b, c]] log2(e)/2 = L L^T; w at the patch centre (0, 0).
    m00 = (0.5 * LOG2E * a).astype(np.float32)
    m01 = (0.5 * LOG2E * b).astype(np.float32)
    m11 = (0.5 * LOG2E * cc).astype(np.float32)
    l11 = np.sqrt(np.maximum(m00, 1e-30)).astype(np.float32)
    l21 = (m01 / l11).astype(np.float32)
    l22 = np.sqrt(np.maximum(m11 - l21 * l21, 1e-30)).astype(np.float32)
    dx, dy = (0.0 - cx).astype(np.float32), (0.0 - cy).astype(np.float32)
    w1e, w2e = (l11 * dx + l21 * dy).astype(np.float32), (l22 * dy).astype(np.float32)
    o = np.log2(opacity).astype(np.float32)
    u = (np.arange(8) - 3.5).astype(F16)
    ux = np.broadcast_to(u[None, None, :], (n, 8, 8))
    uy = np.broadcast_to(u[None, :, None], (n, 8, 8))
    with np.errstate(over="ignore", invalid="ignore"):  # f16 overflow is part of the model
        h = [v.astype(F16)[:, None, None] for v in (l11, l21, l22, w1e, w2e, o)]
        t = fma16(h[0], ux, h[3])
        w1 = fma16(h[1], uy, t)
        w2 = fma16(h[2], uy, h[4])
        p = fma16(-w1, w1, h[5])
        p = fma16(-w2, w2, p).astype(np.float64)
    thr = np.log2(1.0 / 255.0)
    alpha_h = np.where(p >= thr, 2.0 ** np.minimum(p, np.log2(0.99)), 0.0)
    DX = ux.astype(np.float64) - cx[:, None, None]
    DY = uy.astype(np.float64) - cy[:, None, None]
    q = 0.5 * (a[:, None, None] * DX * DX + 2.0 * b[:, None, None] * DX * DY + cc[:, None, None] * DY * DY)
    alpha_e = np.minimum(opacity[:, None, None] * np.exp(-q), 0.99)
    alpha_e = np.where(alpha_e >= 1.0 / 255.0, alpha_e, 0.0)
    return np.abs(alpha_h - alpha_e).reshape(n, -1).max(axis=1)


@pytest.mark.parametrize("filter_variance", [0.3, 0.05])
def test_half2_alpha_error_is_bounded(filter_variance):
    err = model_alpha_error(40000, filter_variance, seed=17)
    assert np.all(np.isfinite(err))
    assert err.max() <= 6e-3, err.max()
    assert np.quantile(err, 0.99) <= 2.5e-3
