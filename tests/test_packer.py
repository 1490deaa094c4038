"""On-device compact packer (gs3d_pack_splats) against the C restatement of
the reference's CPU packer (engine.rs:1801-1891 encode_attributes, compact
layout; spark-lib splat_encode.rs:127-136,234-252; pack_sh engine.rs:1940-1949).

The two sides use different ln/acos/sin implementations (CUDA's and libm), so
a field whose float value sits within an ulp of a quantisation boundary may
land one step apart; the tests require at least 99.9% identical words per
field and at most one step of difference in the others. Means are exact."""
import importlib

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
    assert np.mean(g_sh == o["sh"]) >= 0.999
    L = oracle.lib()
    diff = np.nonzero(g_sh.reshape(-1) != o["sh"].reshape(-1))[0]
    out3 = (np.zeros(3, np.float32), np.zeros(3, np.float32))
    for k in diff[:200]:  # differing words decode within one quantisation step
        for w, buf in zip((g_sh.reshape(-1)[k], o["sh"].reshape(-1)[k]), out3):
            L.gso_decode_sh(int(w), buf.ctypes.data_as(oracle.C.POINTER(oracle.C.c_float)))
        step = np.abs(out3[1]).max() / 127.0 * 2.0
        assert np.abs(out3[0] - out3[1]).max() <= step + 1e-12


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
