"""On-device compact packer (gs3d_pack_splats) against the C restatement of
the reference's CPU packer (engine.rs:1801-1891 encode_attributes, compact
layout; spark-lib splat_encode.rs:127-136,234-252; pack_sh engine.rs:1940-1949).

The two sides use different ln/acos/sin implementations (CUDA's and libm), so
a scale, opacity or rotation field whose float value sits within an ulp of a
quantisation boundary may land one step apart; the tests require at least
99.9% identical words for those and at most one step of difference in the
others. Means and rgb8e8 SH words (no transcendental; the shared exponent
follows the Rust rule, the ceiling of the f32-rounded log2) are identical."""
import importlib
import math

import numpy as np
import pytest

import oracle
from conftest import PKG_NAME

sc = importlib.import_module(PKG_NAME + ".scenes")


def splats(n, degree=3, seed=91):
    rng = np.random.Generator(np.random.PCG64(seed))
    centers = rng.uniform(-50, 50, (n, 3)).astype(np.float32)
    scales = np.exp(rng.normal(-3.0, 1.0, (n, 3))).astype(np.float32)
    opacity = rng.uniform(0.0, 1.0, n).astype(np.float32)
    quats = rng.standard_normal((n, 4)).astype(np.float32)
    rgb = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    C = (degree + 1) ** 2
    rest = (rng.standard_normal((n, C - 1, 3)) * 0.1).astype(np.float32) if degree else None
    return centers, scales, opacity, quats, rgb, rest


def test_f16_conversion_rounds_to_nearest_even_like_numpy():
    L = oracle.lib()
    rng = np.random.Generator(np.random.PCG64(92))
    vals = np.concatenate([
        rng.standard_normal(20000).astype(np.float32) * np.float32(10.0) ** rng.integers(-9, 6, 20000).astype(np.float32),
        np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e10, -1e10, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08,
                  2.9802326e-08, 1.0 + 2 ** -11, 1.0 + 3 * 2 ** -11, np.inf, -np.inf], np.float32)])
    ours = np.array([L.gso_f16_bits(float(v)) for v in vals], np.uint32)
    with np.errstate(over="ignore"):
        ref = vals.astype(np.float16).view(np.uint16).astype(np.uint32)
    assert np.array_equal(ours, ref)


def rounded_log2_ceil(mx: float) -> int:
    """The shared rgb8e8 exponent rule of the device packer (packer.cu):
    ceil of log2 rounded to f32, decided exactly."""
    if math.isnan(mx):
        return 0
    if math.isinf(mx):
        return 127
    f, ex = math.frexp(mx)
    if f == 0.5:
        return ex - 1
    e = ex - 1
    if e == 0:
        return 1
    a = abs(e)
    gap_exp = (a.bit_length() - 1) - 23
    if e < 0 and (a & (a - 1)) == 0:
        gap_exp -= 1
    return e if math.log1p(2.0 * f - 1.0) * 1.4426950408889634074 < math.ldexp(1.0, gap_exp - 1) else e + 1


def near_powers_of_two():
    """f32 values within 48 ulps of every power of two from 2^-126 to 2^127."""
    vals = []
    for e in range(-126, 128):
        base = np.float32(np.ldexp(1.0, e))
        up = base.view(np.uint32) + np.arange(0, 48, dtype=np.uint32)
        down = base.view(np.uint32) - np.arange(1, 48, dtype=np.uint32)
        vals.append(up.view(np.float32))
        vals.append(down.view(np.float32))
    return np.concatenate(vals)


def test_sh_exponent_rule_matches_the_host_log2():
    # The reference computes the exponent as max.log2().ceil() in f32
    # (engine.rs:1945); the oracle restates it with the host's log2f. The
    # device packer's exact decision must agree with it everywhere the two
    # can differ: just above and below each power of two.
    L = oracle.lib()
    vals = near_powers_of_two()
    buf = np.zeros(3, np.float32)
    p = buf.ctypes.data_as(oracle.C.POINTER(oracle.C.c_float))
    for v in vals:
        buf[0] = v
        host = (int(L.gso_pack_sh(p)) >> 24) - 127
        assert host == min(max(rounded_log2_ceil(float(v)), -126), 127), float(v)


def test_cpu_packer_matches_the_numpy_packer():
    centers, scales, opacity, quats, rgb, rest = splats(4000)
    o = oracle.pack_splats(centers, scales, opacity, quats, rgb, rest)
    qn = quats / np.linalg.norm(quats, axis=1, keepdims=True)
    sh_rgb = np.concatenate([((rgb - 0.5) / np.float32(sc.SH_C0))[:, None, :], rest], 1)
    ref = sc.pack_scene(centers, np.zeros(len(centers)), np.log(scales), opacity, qn, sh_rgb)
    assert np.array_equal(o["means"], ref["means"])
    assert np.mean(o["shape"] == ref["shape"]) >= 0.999
    assert np.mean(o["rotations"] == ref["rotations"]) >= 0.999
    assert np.mean(o["sh"].reshape(-1) == ref["sh"][: o["sh"].size]) >= 0.999


@pytest.mark.gpu
@pytest.mark.parametrize("degree", [0, 1, 3])
def test_device_packer_matches_the_cpu_packer(degree):
    import torch
    P = importlib.import_module(PKG_NAME)
    n, first, capacity = 20000, 37, 20100
    centers, scales, opacity, quats, rgb, rest = splats(n, degree, seed=93 + degree)
    o = oracle.pack_splats(centers, scales, opacity, quats, rgb, rest, object_id=5)
    C = (degree + 1) ** 2
    t = {k: torch.from_numpy(v).cuda() for k, v in dict(c=centers, s=scales, o=opacity, q=quats, r=rgb).items()}
    rest_t = torch.from_numpy(rest).cuda() if rest is not None else None
    means = torch.zeros((capacity, 4), dtype=torch.float32, device="cuda")
    shape = torch.zeros((capacity, 2), dtype=torch.int32, device="cuda")
    rot = torch.zeros(capacity, dtype=torch.int32, device="cuda")
    sh = torch.zeros(capacity * C + capacity, dtype=torch.int32, device="cuda")
    P.pack_splats(t["c"], t["s"], t["o"], t["q"], t["r"], rest_t, first, means, shape, rot, sh, capacity, object_id=5)
    torch.cuda.synchronize()
    g_means = means.cpu().numpy()[first:first + n]
    g_shape = shape.cpu().numpy().view(np.uint32)[first:first + n]
    g_rot = rot.cpu().numpy().view(np.uint32)[first:first + n]
    g_sh = sh.cpu().numpy().view(np.uint32)[first * C:(first + n) * C].reshape(n, C)
    assert np.array_equal(g_means.view(np.uint32), o["means"].view(np.uint32))
    # Untouched slots stay zero.
    assert not means.cpu().numpy()[:first].any() and not means.cpu().numpy()[first + n:].any()
    for g, c, fields in ((g_shape, o["shape"], ((0, 16), (16, 16))),
                         (g_rot, o["rotations"], ((0, 10), (10, 10), (20, 12)))):
        assert np.mean(g == c) >= 0.999
        for lo, bits in fields:
            fg = (g >> lo) & ((1 << bits) - 1)
            fc = (c >> lo) & ((1 << bits) - 1)
            assert np.abs(fg.astype(np.int64) - fc.astype(np.int64)).max() <= 1
    # SH words involve no transcendental on either side: identical.
    assert np.array_equal(g_sh, o["sh"])


@pytest.mark.gpu
def test_device_sh_exponent_near_powers_of_two():
    # Coefficients within 48 ulps of every power of two: the device's exact
    # exponent decision equals the restatement's f32 log2 word for word.
    import torch
    P = importlib.import_module(PKG_NAME)
    vals = near_powers_of_two()
    vals = vals[np.abs(vals) < 1e30]  # keep (rgb - 0.5) / SH_C0 and the rest finite
    n = vals.size // 3
    v = vals[: 3 * n].reshape(n, 3)
    rng = np.random.Generator(np.random.PCG64(96))
    v = v * np.where(rng.random((n, 3)) < 0.5, -1, 1).astype(np.float32)
    centers = np.zeros((n, 3), np.float32)
    scales = np.full((n, 3), 0.01, np.float32)
    opacity = np.full(n, 0.5, np.float32)
    quats = np.tile(np.array([0, 0, 0, 1], np.float32), (n, 1))
    rgb = np.full((n, 3), 0.5, np.float32)
    rest = np.repeat(v[:, None, :], 3, axis=1)  # degree 1: three rest coefficients
    o = oracle.pack_splats(centers, scales, opacity, quats, rgb, rest)
    t = [torch.from_numpy(a).cuda() for a in (centers, scales, opacity, quats, rgb, rest)]
    means = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    shape = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    rot = torch.zeros(n, dtype=torch.int32, device="cuda")
    sh = torch.zeros(n * 4 + n, dtype=torch.int32, device="cuda")
    P.pack_splats(*t, 0, means, shape, rot, sh, n)
    torch.cuda.synchronize()
    g_sh = sh.cpu().numpy().view(np.uint32)[: n * 4].reshape(n, 4)
    assert np.array_equal(g_sh, o["sh"])


@pytest.mark.gpu
def test_device_packed_scene_renders_like_the_host_packed_scene():
    import torch
    P = importlib.import_module(PKG_NAME)
    dev = importlib.import_module(PKG_NAME + ".device")
    from gpu_harness import GpuRun, psnr
    n = 8000
    rng = np.random.Generator(np.random.PCG64(95))
    centers = rng.uniform(-4, 4, (n, 3)).astype(np.float32)
    scales = np.exp(rng.normal(-2.6, 0.5, (n, 3))).astype(np.float32)
    opacity = (1 / (1 + np.exp(-rng.normal(0, 1.5, n)))).astype(np.float32)
    quats = rng.standard_normal((n, 4)).astype(np.float32)
    rgb = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    rest = (rng.standard_normal((n, 15, 3)) * 0.1).astype(np.float32)
    qn = quats / np.linalg.norm(quats, axis=1, keepdims=True)
    host = sc.pack_scene(centers, np.zeros(n), np.log(scales), opacity, qn,
                         np.concatenate([((rgb - 0.5) / np.float32(sc.SH_C0))[:, None, :], rest], 1))
    frame = sc.make_frame(sc.look_at((0, 1, 12), (0, 0, 0)), 320, 200, 55.0, 0.1, 100.0)
    run = GpuRun(host, frame, "fp32")
    ref = run.render(frame)
    run.close()
    packed = dict(host)
    t = [torch.from_numpy(a).cuda() for a in (centers, scales, opacity, quats, rgb, rest)]
    means = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    shape = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    rot = torch.zeros(n, dtype=torch.int32, device="cuda")
    sh = torch.zeros(n * 16 + n, dtype=torch.int32, device="cuda")
    sh[n * 16:] = torch.arange(n, dtype=torch.int32, device="cuda")  # active-slot tail
    P.pack_splats(*t, 0, means, shape, rot, sh, n)
    torch.cuda.synchronize()
    packed.update(means=means.cpu().numpy(), shape=shape.cpu().numpy().view(np.uint32),
                  rotations=rot.cpu().numpy().view(np.uint32), sh=sh.cpu().numpy().view(np.uint32))
    run = GpuRun(packed, frame, "fp32")
    g = run.render(frame)
    run.close()
    assert psnr(g["rgba"][..., :3], ref["rgba"][..., :3]) >= 60.0
    assert abs(int(g["visible_state"][0]) - int(ref["visible_state"][0])) <= 2
