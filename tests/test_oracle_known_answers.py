"""The oracle against the reference's own known-answer tests.

Each case restates a vector from the reference test suite (file:line cited)
and checks the CPU oracle with the same tolerance the reference test uses
(vitest ``toBeCloseTo(v, d)`` means |x - v| < 10^-d / 2).
"""
import json
import math
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")


def close(x, v, digits):
    return abs(x - v) < 10 ** (-digits) / 2


@pytest.fixture(scope="module")
def L():
    return oracle.lib()


@pytest.fixture(scope="module")
def kat():
    with open(GOLDEN) as f:
        return json.load(f)


def proj_cov(L, scale, rot, mv):
    out = oracle.out_f32(9)
    L.gso_view_covariance(oracle.f32(scale), oracle.f32(rot), oracle.f32(mv), out)
    return np.array(out[:], np.float32)


def perspective(L, view, cov9, proj, vp, filt):
    out = oracle.out_f32(16)
    L.gso_perspective_projection(oracle.f32(view), oracle.f32(cov9), oracle.f32(proj),
                                 oracle.f32(vp), filt, out)
    return np.array(out[:], np.float32).reshape(4, 4)  # rows are WGSL columns


def valid(L, p):
    return L.gso_projection_is_valid(oracle.f32(np.asarray(p, np.float32).ravel()))


def test_default_perspective_projection(L, kat):
    # test/ProjectionBoundary.test.ts:30-54
    c = kat["perspective_default"]
    eye = np.eye(4, dtype=np.float32).T.ravel()
    cov = proj_cov(L, [1, 1, 1], [0, 0, 0, 1], eye)
    p = perspective(L, c["view"], cov, eye, c["viewport"], c["filter"])
    assert list(p[0, :3]) == c["center_depth"]
    assert close(p[2, 0], c["cov_xx"], 4)
    assert close(p[1, 0], 1 / c["cov_xx"], 6)
    assert p[2, 3] == c["unfiltered_det"]
    assert valid(L, p) == 1
    clipped = perspective(L, c["clipped_view"], cov, eye, c["viewport"], c["filter"])
    assert clipped[0, 3] == 0


def test_unfiltered_projection_and_rejections(L, kat):
    # test/ProjectionBoundary.test.ts:56-72
    c = kat["projection_result"]
    out = oracle.out_f32(16)
    L.gso_projection_result(oracle.f32(c["center"]), c["depth"], oracle.f32(c["cov"]), 0.0, out)
    p = np.array(out[:], np.float32).reshape(4, 4)
    assert p[0, 2] == c["depth"] and p[2, 0] == c["cov"][0]
    assert close(p[2, 2], c["cov"][2], 4)
    assert valid(L, p) == 1
    neg = p.copy(); neg[0, 2] = -1.0
    inf = p.copy(); inf[0, 2] = np.inf
    bad = p.copy(); bad[1, 0] = 99.0
    assert [valid(L, neg), valid(L, inf), valid(L, bad)] == [0, 0, 0]


@pytest.mark.parametrize("axis", [1, 2])
def test_periodic_delta_picks_strongest_image(L, kat, axis):
    # test/ProjectionBoundary.test.ts:74-104
    c = kat["periodic_delta"]
    conic, vp, center = c["conic"], c["viewport"], c["center"]
    for pixel in c["pixels"]:
        out = oracle.out_f32(2)
        L.gso_boundary_delta(oracle.f32(pixel), oracle.f32(center), oracle.f32(conic),
                             oracle.f32(vp), axis, out)
        power = lambda x, y: conic[0] * x * x + 2 * conic[1] * x * y + conic[2] * y * y
        actual = power(out[0], out[1])
        best = min(power(pixel[0] - center[0] - (i * vp[0] if axis == 1 else 0),
                         pixel[1] - center[1] - (i * vp[1] if axis == 2 else 0))
                   for i in range(-100, 101))
        assert close(actual, best, 4)


@pytest.mark.parametrize("idx", range(4))
def test_tile_hits_are_counted_once_and_conservative(L, kat, idx):
    # test/ProjectionBoundary.test.ts:106-163
    fx = kat["tile_hit_fixtures"][idx]
    center, cov, W, H, axis = fx["center"], fx["cov"], fx["width"], fx["height"], fx["axis"]
    det = cov[0] * cov[2] - cov[1] * cov[1]
    conic = [cov[2] / det, -cov[1] / det, cov[0] / det]
    thr = math.log(255)
    radius = [math.ceil(math.sqrt(2 * thr * cov[0])), math.ceil(math.sqrt(2 * thr * cov[2]))]
    nx, ny = math.ceil(W / 16), math.ceil(H / 16)
    args = (oracle.f32(center), oracle.f32(conic), thr, oracle.f32(radius))
    hits = [L.gso_boundary_tile_hit(*args, t % nx, t // nx, oracle.f32([W, H]), axis)
            for t in range(nx * ny)]
    count = L.gso_count_tiles(*args, 0, 0, nx - 1, ny - 1, oracle.f32([W, H]), axis)
    assert count == sum(hits)
    assert count <= nx * ny
    sampled = 0
    for y in range(H):
        for x in range(W):
            best = min(0.5 * (conic[0] * dx * dx + 2 * conic[1] * dx * dy + conic[2] * dy * dy)
                       for i in range(-100, 101)
                       for dx, dy in [(x + 0.5 - center[0] - (i * W if axis == 1 else 0),
                                       y + 0.5 - center[1] - (i * H if axis == 2 else 0))])
            if best <= thr:
                sampled += 1
                assert hits[(y // 16) * nx + (x // 16)] == 1
    assert sampled > 0


def test_periodic_subpixel_sample(L, kat):
    # test/ProjectionBoundary.test.ts:165-175
    c = kat["subpixel"]
    r = [L.gso_subpixel_has_sample(oracle.f32(c["center"]), oracle.f32(c["conic"]), c["thr"],
                                   oracle.f32(c["extent"]), c["viewport"][0], c["viewport"][1], axis)
         for axis in (1, 0)]
    assert r == c["expected"]


def test_depth_finalisation(L, kat):
    # test/ScalarOutput.test.ts:61-97 (raw scalar encoding, alpha threshold 0.5,
    # invalid value Infinity)
    c = kat["finalize_depth"]
    inf = float("inf")
    fin = lambda w, t: L.gso_finalize_depth(w, t, 0.1, 1000.0, 0.5, inf, 1)
    assert all(fin(w, t) == inf for w, t in c["invalid"])
    a, b = (fin(w, t) for w, t in c["finite"])
    assert close(a, c["finite_expected"][0], 5) and close(b, c["finite_expected"][1], 3)
    # accumulated coverage 0.1 below the 0.5 threshold is invalid whatever the encoding
    assert fin(0.1, 0.9) == inf
    # device-depth encoding of the default node: clamp((n + z) f / ((f - n) z), 0, 1)
    d = L.gso_finalize_depth(8.8, 0.2, 1.0, 100.0, 0.5, inf, 0)
    z = -11.0
    assert abs(d - (1.0 + z) * 100.0 / ((100.0 - 1.0) * z)) < 1e-6


def test_sh_rgb8e8_round_trip(L, kat):
    # test/GaussianSh.test.ts:19-41 (packer: rust/gaussian-backend/src/engine.rs:1940-1949)
    for rgb in kat["sh_round_trip"]:
        word = L.gso_pack_sh(oracle.f32(rgb))
        out = oracle.out_f32(3)
        L.gso_decode_sh(word, out)
        mx = max(abs(v) for v in rgb)
        tol = 0 if mx == 0 else 2 ** math.ceil(math.log2(mx)) / 127
        for ch in range(3):
            assert abs(out[ch] - rgb[ch]) <= tol + 2.220446049250313e-16


def test_compact_geometry_precision(L, kat):
    # rust/gaussian-backend/tests/backend.rs:1086-1174: compact shape within 1 %,
    # opacity within 1e-3, quaternion |dot| > 0.99999.
    import importlib
    sc = importlib.import_module("3dgs_tile_webgpu_gb300.scenes")
    for case in kat["compact_geometry"]:
        scale = np.array(case["scale"], np.float64)
        q = np.array(case["quat"], np.float32)
        op = case["opacity"]
        ls = np.log(scale).astype(np.float32)
        packed = sc.pack_scene(np.array([case["position"]], np.float32), [0], ls[None], [op],
                               q[None], np.zeros((1, 1, 3), np.float32))
        x, y = (int(v) for v in packed["shape"][0])
        out = oracle.out_f32(4)
        L.gso_decode_scale_opacity(x, y, out)
        for axis in range(3):
            assert abs(out[axis] / scale[axis] - 1.0) < 0.01
        assert abs(out[3] - op) < 1e-3
        L.gso_decode_rotation(int(packed["rotations"][0]), out)
        assert abs(float(np.dot(np.array(out[:]), q))) > 0.99999
        # the oracle's own encoder agrees with the numpy packer
        assert L.gso_encode_oct101012(oracle.f32(q)) == int(packed["rotations"][0])
        # means stay float32 exactly (123456.75 survives)
        assert packed["means"][0, 0] == np.float32(case["position"][0])


def test_chunk_composite_matches_whole_stream(kat):
    # test/rasterizationWGSL.test.ts:63-86: ordered chunk composite equals the
    # whole alpha stream.
    samples = kat["chunk_composite"]

    def comp(s):
        col, t = [0.0, 0.0, 0.0], 1.0
        for smp in s:
            for ch in range(3):
                col[ch] += smp["color"][ch] * t * smp["alpha"]
            t *= 1 - smp["alpha"]
        return col, t

    whole = comp(samples)
    a, b = comp(samples[:2]), comp(samples[2:])
    col = [a[0][ch] + a[1] * b[0][ch] for ch in range(3)]
    for ch in range(3):
        assert close(col[ch], whole[0][ch], 12)
    assert close(a[1] * b[1], whole[1], 12)


def test_tile_sort_bits(L):
    # TiledGaussianPipeline.ts:431,442-446: 13 bits at 1280x720, 14 at 1080p, 16 at 4K.
    assert L.gso_tile_sort_bits(80 * 45) == 13
    assert L.gso_tile_sort_bits(120 * 68) == 14
    assert L.gso_tile_sort_bits(240 * 135) == 16


def test_oracle_chunked_raster_composites_to_the_whole_stream():
    # The same rule through the oracle's own rasterizer: with chunks of 256
    # samples (TileRasterizer.ts:807-902, rasterChunks.ts:3-99) every tile
    # of more than 256 records is blended as ordered chunk partials and
    # composited; with chunking off it is one stream. In the FP64 twin, and
    # with a transmittance threshold too small to stop any pixel early (the
    # early stop is the one place the two differ by design), the images agree
    # to rounding.
    from conftest import scenes
    sc = scenes()
    scene = sc.uniform_cloud(8000, seed=17, log_scale=(-1.6, 0.4), opacity_logit=(-2.0, 0.5))
    base = sc.make_frame(sc.look_at((0.5, 1.0, 11.0), (0, 0, 0)), 64, 48, 55.0, 0.1, 100.0,
                         transmittance_threshold=1e-30)
    whole = oracle.render(scene, dict(base, raster_chunk_size=0), 1)
    chunked = oracle.render(scene, dict(base, raster_chunk_size=256), 1)
    loads = np.diff(whole["tile_offsets"].astype(np.int64))
    assert loads.max() > 2 * 256  # some tiles split into three or more chunks
    assert np.array_equal(whole["sorted_records"], chunked["sorted_records"])
    assert np.abs(whole["rgba"] - chunked["rgba"]).max() <= 1e-9
    # In FP32 the two orders of the same sums round differently: the chunked
    # path did run, and stays within rounding of the whole stream.
    whole32 = oracle.render(scene, dict(base, raster_chunk_size=0), 0)
    chunked32 = oracle.render(scene, dict(base, raster_chunk_size=256), 0)
    diff = np.abs(whole32["rgba"] - chunked32["rgba"]).max()
    assert 0.0 < diff <= 1e-5
