"""Tile size as a launch-shape knob of batched renders (gs3d_tuning.tile_size).

The reference fixes its tiles at 16x16 pixels (src/renderer/pipeline/constants.ts:1).
Batched renders here may also use 8x8 or 32x32 tiles; the rasterizer's block
follows the tile. What each pixel sees does not change: a splat that fails
the reference's tile test for a tile (tileContribution.ts:16-59, the minimum
of its quadratic over the tile) fails the per-pixel test at every pixel of
that tile, and the records of a tile keep the (depth, ordinal) order. So the
EXACT image is the same bits at every tile size (cases with neither a raster
chunk split nor a per-tile cap, which act per tile) and the per-tile buffers
keep their invariants. The visible set may differ, but only by splats whose
support reaches a tile only in the part of it past the image edge (a 120-row
image has a last row of 16-pixel tiles reaching row 128, of 8-pixel tiles
row 120): they cover no pixel.
"""
import importlib

import numpy as np
import pytest

import oracle
from conftest import PKG_NAME, scenes
from gpu_harness import psnr, render_batch
from test_gpu_parity import CASES

pytestmark = pytest.mark.gpu

sc = scenes()
P = importlib.import_module(PKG_NAME)

# Cases whose tiles are never split into raster chunks and carry no cap.
SAME_IMAGE_CASES = sorted(set(CASES) - {"capped", "chunked"})


CAMERA_KEYS = ("projection", "view", "width", "height", "near", "far", "objects")


def batch_of(name):
    """The parity case's view and a second view of the same scene (another
    camera and size, the same pass options): one view group."""
    scene, frame = CASES[name]()
    opts = {k: v for k, v in frame.items() if k not in CAMERA_KEYS}
    second = sc.make_frame(sc.look_at((-2.0, 1.5, 10.5), (0, 0, 0)), 128, 80, 55.0, 0.1, 100.0, **opts)
    return [(scene, frame), (scene, second)]


@pytest.mark.parametrize("name", SAME_IMAGE_CASES)
def test_exact_image_is_the_same_at_every_tile_size(name):
    pairs = batch_of(name)
    ref, _ = render_batch(pairs, "exact", share_scenes=True)
    for tile in (8, 32):
        got, _ = render_batch(pairs, "exact", share_scenes=True, tuning={"tile_size": tile})
        for (_, frame), g, r in zip(pairs, got, ref):
            assert np.array_equal(g["rgba"].view(np.uint32), r["rgba"].view(np.uint32)), tile
            assert np.array_equal(g["depth"].view(np.uint32), r["depth"].view(np.uint32)), tile
            # A splat visible at one tile size only has all its records in
            # that size's partial edge tiles (the ones reaching past the image).
            a, b = set(g["depth_sorted"][:, 1].tolist()), set(r["depth_sorted"][:, 1].tolist())
            assert len(a ^ b) <= 0.01 * len(b) + 16
            for ordinal in a ^ b:
                res, ts = (g, tile) if ordinal in a else (r, 16)
                W, H = int(frame["width"]), int(frame["height"])
                tiles_x = (W + ts - 1) // ts
                recs = res["sorted_records"]
                for t in recs[recs[:, 1] == ordinal, 0]:
                    tx, ty = int(t) % tiles_x, int(t) // tiles_x
                    edge_x = W % ts != 0 and tx == tiles_x - 1
                    edge_y = H % ts != 0 and ty == (H + ts - 1) // ts - 1
                    assert edge_x or edge_y, (ordinal, ts, tx, ty)
    # The 16-pixel batch is the reference's: equal to the oracle's image.
    for (scene, frame), r in zip(pairs, ref):
        o = oracle.render(scene, frame, 0)
        assert np.array_equal(r["rgba"].view(np.uint32), o["rgba"].view(np.uint32))


@pytest.mark.parametrize("tile", [8, 32])
def test_per_tile_buffers_keep_their_invariants(tile):
    scene, frame = CASES["default"]()
    pairs = [(scene, frame), (sc.uniform_cloud(3000, seed=81, log_scale=(-2.0, 0.5)),
                              sc.make_frame(sc.look_at((1.0, 2.0, 9.0), (0, 0, 0)), 97, 64, 55.0, 0.1, 100.0))]
    views, _ = render_batch(pairs, "exact", tuning={"tile_size": tile})
    for (s, f), g in zip(pairs, views):
        W, H = int(f["width"]), int(f["height"])
        ntile = ((W + tile - 1) // tile) * ((H + tile - 1) // tile)
        recs = g["sorted_records"]
        assert g["tile_offsets"].size == ntile + 1
        assert recs.shape[0] == int(g["tile_counts"].sum()) > 0
        assert np.all(recs[:, 0] < ntile)
        keys = g["proj_mean"][:, 2].view(np.uint32)
        order = np.lexsort((recs[:, 1], keys[recs[:, 1]], recs[:, 0]))
        assert np.array_equal(order, np.arange(recs.shape[0]))  # (tile, depth key, ordinal)
        assert np.array_equal(np.bincount(recs[:, 1], minlength=g["tile_counts"].size), g["tile_counts"])
        assert np.array_equal(g["tile_offsets"], np.searchsorted(recs[:, 0], np.arange(ntile + 1)))


@pytest.mark.parametrize("precision", ["half2", "fp32"])
@pytest.mark.parametrize("tile", [8, 32])
def test_fast_forms_at_other_tile_sizes(precision, tile):
    # Each batch shares one set of pass options (those of its first view).
    for name in ("default", "repeat_x"):
        pairs = batch_of(name)
        ref, _ = render_batch(pairs, precision, share_scenes=True)
        got, _ = render_batch(pairs, precision, share_scenes=True, tuning={"tile_size": tile})
        for (scene, frame), g, r in zip(pairs, got, ref):
            o64 = oracle.render(scene, frame, 1)
            assert np.abs(g["rgba"] - r["rgba"]).max() <= 2e-2, name
            assert psnr(g["rgba"][..., :3], o64["rgba"][..., :3]) >= 50.0, name


def test_graph_replay_at_tile_8_matches_direct_batches():
    import torch
    dev = importlib.import_module(PKG_NAME + ".device")
    ds = dev.DeviceScene(sc.uniform_cloud(5000, seed=82, log_scale=(-2.4, 0.6)))
    sizes = [(200, 120), (97, 64)]
    frames = [sc.make_frame(sc.look_at((x, 1.0, 11.0), (0, 0, 0)), w, h, 55.0, 0.1, 100.0)
              for x, (w, h) in zip((-1.0, 1.5), sizes)]
    colors = [torch.zeros((h, w, 4), dtype=torch.float16, device="cuda") for (w, h) in sizes]
    refs = [torch.zeros_like(c) for c in colors]
    graph = P.TiledGaussianPipeline(ds.data(), {"raster_precision": "half2", "intersection_capacity": 1 << 20})
    direct = P.TiledGaussianPipeline(ds.data(), {"raster_precision": "half2", "intersection_capacity": 1 << 20})
    graph.set_tuning({"tile_size": 8})
    direct.set_tuning({"tile_size": 8})
    cams = [P.make_camera(f) for f in frames]
    stream = torch.cuda.Stream()
    graph.capture_graph([(ds.data(), c, w, h, col.data_ptr(), 0, "rgba16f")
                         for c, (w, h), col in zip(cams, sizes, colors)], stream.cuda_stream)
    for step in range(3):
        fr = [sc.make_frame(sc.look_at((step - 1.0, 1.0 + step, 11.0), (0, 0, 0)), w, h, 55.0, 0.1, 100.0)
              for (w, h) in sizes]
        cams = [P.make_camera(f) for f in fr]
        graph.launch_graph(cams, attempt=step + 1, stream=stream.cuda_stream)
        stream.synchronize()
        direct.render_batch([(ds.data(), c, w, h, col.data_ptr(), 0, "rgba16f")
                             for c, (w, h), col in zip(cams, sizes, refs)], attempt=step + 1)
        torch.cuda.synchronize()
        for a, b in zip(colors, refs):
            assert torch.equal(a, b), step
    graph.dispose()
    direct.dispose()


def test_invalid_tile_size_is_rejected():
    dev = importlib.import_module(PKG_NAME + ".device")
    ds = dev.DeviceScene(sc.uniform_cloud(1000, seed=83))
    pipe = P.TiledGaussianPipeline(ds.data(), {"intersection_capacity": 1 << 16})
    for bad in (4, 12, 64):
        with pytest.raises(ValueError):
            pipe.set_tuning({"tile_size": bad})
    pipe.set_tuning({"tile_size": 0})
    assert pipe.get_tuning()["tile_size"] == 16
    pipe.dispose()


@pytest.mark.parametrize("precision", ["half2", "fp32"])
@pytest.mark.parametrize("name", ["default", "repeat_y", "chunked", "capped", "background_depth_raw"])
def test_four_pixels_per_lane(precision, name):
    # The fast rasterizers' other block shape (a warp per 8x16 patch, four
    # pixels per lane): the image stays within the fast forms' tolerance of
    # the two-pixel shape and of the oracle, at 16- and 32-pixel tiles (16
    # only where a per-tile cap applies).
    pairs = batch_of(name)
    ref, _ = render_batch(pairs, precision, share_scenes=True)
    # maxRasterizedSplatsPerTile acts per tile: the capped case keeps 16.
    for tile in ((16,) if name == "capped" else (16, 32)):
        got, _ = render_batch(pairs, precision, share_scenes=True,
                              tuning={"tile_size": tile, "raster_pixels_per_lane": 4})
        for (scene, frame), g, r in zip(pairs, got, ref):
            o = oracle.render(scene, frame, 0)
            o64 = oracle.render(scene, frame, 1)
            assert np.abs(g["rgba"] - r["rgba"]).max() <= 2e-2, tile
            assert np.abs(g["rgba"] - o["rgba"]).max() <= 2e-2, tile
            assert psnr(g["rgba"][..., :3], o64["rgba"][..., :3]) >= 50.0, tile
            if name == "background_depth_raw":
                # The depth is the invalid value below the coverage threshold
                # (finalizeGaussianDepth.ts): pixels whose coverage lies within
                # the colour tolerance of it may fall on either side.
                bga = frame["background"][3]
                cover = 1.0 - (1.0 - r["rgba"][..., 3]) / (1.0 - bga)
                steady = np.abs(cover - frame["depth_alpha_threshold"]) > 2e-2
                finite = np.isfinite(r["depth"]) & np.isfinite(g["depth"]) & steady
                assert np.abs(g["depth"][finite] - r["depth"][finite]).max() <= 2e-2 * max(1.0, np.abs(r["depth"][finite]).max())


def test_four_pixels_per_lane_counts_the_same_work():
    # rasterStats with the other block shape: the same pixels, and the
    # checked / blended samples within the regrouping of the transmittance
    # test (at most 31 records per pixel past the exact stop).
    import torch
    dev = importlib.import_module(PKG_NAME + ".device")
    scene, frame = CASES["default"]()
    ds = dev.DeviceScene(scene)
    W, H = int(frame["width"]), int(frame["height"])
    out = {}
    for ppl in (2, 4):
        pipe = P.TiledGaussianPipeline(ds.data(), {"raster_precision": "half2", "raster_stats": True,
                                                   "intersection_capacity": 1 << 20})
        pipe.set_tuning({"raster_pixels_per_lane": ppl})
        color = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        pipe.render_batch([(ds.data(), P.make_camera(frame), W, H, color.data_ptr(), 0, "rgba32f")])
        out[ppl] = pipe.read_stats()["rasterWork"]
        pipe.dispose()
    assert out[4]["pixels"] == out[2]["pixels"] > 0
    for k in ("checked", "blended"):
        assert abs(out[4][k] - out[2][k]) <= 31 * out[2]["pixels"], k
        assert out[4][k] > 0


def test_invalid_pixels_per_lane_is_rejected():
    dev = importlib.import_module(PKG_NAME + ".device")
    ds = dev.DeviceScene(sc.uniform_cloud(1000, seed=84))
    pipe = P.TiledGaussianPipeline(ds.data(), {"intersection_capacity": 1 << 16})
    for bad in (1, 3, 8):
        with pytest.raises(ValueError):
            pipe.set_tuning({"raster_pixels_per_lane": bad})
    pipe.set_tuning({"raster_pixels_per_lane": 0})
    assert pipe.get_tuning()["raster_pixels_per_lane"] == 2
    pipe.dispose()
