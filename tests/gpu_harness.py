"""Runs the CUDA pass through the C ABI and fetches every intermediate buffer,
for comparison with the CPU oracle (test helper)."""
import importlib

import numpy as np

from conftest import PKG_NAME

P = importlib.import_module(PKG_NAME)
dev = importlib.import_module(PKG_NAME + ".device")


def pipeline_options(frame: dict, precision: str = "exact", capacity: int | None = None) -> dict:
    return {
        "intersection_capacity": int(capacity if capacity is not None else frame.get("capacity", 1 << 22)),
        "raster_chunk_size": int(frame.get("raster_chunk_size", 8192)),
        "background": tuple(frame.get("background", (0, 0, 0, 0))),
        "depth_sort_mode": "packed16" if frame.get("depth_sort_mode", 0) == 1 else "float32",
        "antialias_mode": "classic" if frame.get("antialias", 0) == 1 else "compensated",
        "boundary_policy": {0: "clip", 1: "repeat-x", 2: "repeat-y"}[int(frame.get("boundary_axis", 0))],
        "subpixel_sample_culling": bool(frame.get("subpixel_culling", 1)),
        "max_rasterized_splats_per_tile": int(frame.get("max_splats_per_tile", 0)) or None,
        "raster_transmittance_threshold": float(frame.get("transmittance_threshold", 1e-4)),
        "depth_alpha_threshold": float(frame.get("depth_alpha_threshold", 0.95)),
        "filter_variance": float(frame.get("filter_variance", 0.3)),
        "invalid_depth_value": float(frame.get("invalid_depth_value", 1.0)),
        "depth_encoding": "raw" if frame.get("depth_encoding", 0) == 1 else "device",
        "raster_precision": precision,
        "projection_precision": frame.get("projection_precision", "fp32"),
    }


class GpuRun:
    """One pipeline over one resident scene; render() fetches everything."""

    def __init__(self, scene: dict, frame: dict, precision: str = "exact", capacity: int | None = None):
        self.ds = dev.DeviceScene(scene)
        self.pipe = P.TiledGaussianPipeline(self.ds.data(), pipeline_options(frame, precision, capacity))

    def render(self, frame: dict, color_format: str = "rgba32f", attempt: int = 1, reset_valid: bool = False,
               color_init: float | None = None) -> dict:
        import torch
        W, H = int(frame["width"]), int(frame["height"])
        self.pipe.prepare_frame(W, H)
        dtype = torch.float16 if color_format == "rgba16f" else torch.float32
        color = torch.zeros((H, W, 4), dtype=dtype, device="cuda")
        if color_init is not None:
            color.fill_(color_init)
        depth = torch.zeros((H, W), dtype=torch.float32, device="cuda")
        self.pipe.render(P.make_camera(frame), color.data_ptr(), depth.data_ptr(), attempt, reset_valid,
                         color_format)
        stats = self.pipe.read_stats()
        r = self.pipe.get_resources()
        n = int(self.ds.active_count)
        out = {"stats": stats, "launches": self.pipe.last_launch_count()}
        vis = dev.to_numpy(r.visible_state, (4,))
        state = dev.to_numpy(r.dispatch_state, (4,))
        V, cnt = int(vis[0]), int(state[0])
        ntile = int(r.tiles_x) * int(r.tiles_y)
        out["visible_state"], out["state"] = vis, state
        out["output_state"] = dev.to_numpy(r.output_state, (4,))
        out["proj_mean"] = dev.to_numpy(r.projected_mean, (n, 4), np.float32)
        out["proj_conic"] = dev.to_numpy(r.projected_conic, (n, 4), np.float32)
        out["proj_color"] = dev.to_numpy(r.projected_color, (n, 4), np.float32)
        out["tile_counts"] = dev.to_numpy(r.tile_counts, (n,))
        out["visible_offsets"] = dev.to_numpy(r.visible_offsets, (n,))
        out["depth_sorted"] = np.stack([dev.to_numpy(r.depth_sorted_keys, (V,)),
                                        dev.to_numpy(r.depth_sorted_ids, (V,))], 1)
        out["ordered_counts"] = dev.to_numpy(r.depth_ordered_tile_counts, (V,))
        out["intersection_offsets"] = dev.to_numpy(r.intersection_offsets, (V,))
        out["sorted_records"] = np.stack([dev.to_numpy(r.sorted_tile_ids, (cnt,)),
                                          dev.to_numpy(r.sorted_gaussian_ids, (cnt,))], 1)
        out["tile_offsets"] = dev.to_numpy(r.tile_offsets, (ntile + 1,))
        assert int(r.total_tiles) == ntile
        out["rgba"] = color.float().cpu().numpy()
        out["depth"] = depth.cpu().numpy()
        return out

    def close(self):
        self.pipe.dispose()


# The fast raster forms evaluate the SH colour with fused multiply-adds (the
# colour feeds only their image): projected colours within this of the
# oracle's, the slot tag in the fourth component still exact.
FAST_COLOR_TOL = 1e-5


def assert_bit_exact(g: dict, o: dict, image: bool = True, color_tol: float = 0.0) -> None:
    """Every buffer the reference exposes through getResources() is identical
    (the projected colour within color_tol when it is nonzero)."""
    assert np.array_equal(g["visible_state"], o["visible_state"]), (g["visible_state"], o["visible_state"])
    assert np.array_equal(g["tile_counts"], o["tile_counts"])
    assert np.array_equal(g["proj_mean"].view(np.uint32), o["proj_mean"].view(np.uint32))
    vis = o["tile_counts"] > 0
    assert np.array_equal(g["proj_conic"][vis].view(np.uint32), o["proj_conic"][vis].view(np.uint32))
    if color_tol:
        assert np.abs(g["proj_color"][vis][:, :3] - o["proj_color"][vis][:, :3]).max(initial=0.0) <= color_tol
        assert np.array_equal(g["proj_color"][vis][:, 3].view(np.uint32), o["proj_color"][vis][:, 3].view(np.uint32))
    else:
        assert np.array_equal(g["proj_color"][vis].view(np.uint32), o["proj_color"][vis].view(np.uint32))
    assert np.array_equal(g["visible_offsets"], o["visible_offsets"])
    assert np.array_equal(g["depth_sorted"], o["depth_sorted"])
    assert np.array_equal(g["ordered_counts"], o["ordered_counts"])
    assert np.array_equal(g["intersection_offsets"], o["intersection_offsets"])
    assert np.array_equal(g["state"], o["state"]), (g["state"], o["state"])
    assert np.array_equal(g["output_state"], o["output_state"]), (g["output_state"], o["output_state"])
    assert np.array_equal(g["sorted_records"], o["sorted_records"])
    assert np.array_equal(g["tile_offsets"], o["tile_offsets"])
    if image:
        assert np.array_equal(g["rgba"].view(np.uint32), o["rgba"].view(np.uint32))
        assert np.array_equal(g["depth"].view(np.uint32), o["depth"].view(np.uint32))


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(1.0 / mse)


def render_batch(scenes_frames: list, precision: str = "exact", capacity: int = 1 << 22,
                 color_format: str = "rgba32f", share_scenes: bool = False, tuning: dict | None = None) -> list:
    """Render (scene, frame) pairs in one batch and split every buffer per view.

    Each view's result uses the view's own ordinals and local tile ids, so it
    compares directly with a single-view oracle render of that view (at the
    tuning's tile size: the reference's 16 unless `tuning` sets another). With
    share_scenes, pairs holding the same scene object render from one resident
    copy (one set of device buffers), so consecutive ones form a view group."""
    import torch
    if share_scenes:
        resident = {}
        dss = [resident.setdefault(id(s), dev.DeviceScene(s)) if id(s) not in resident else resident[id(s)]
               for s, _ in scenes_frames]
    else:
        dss = [dev.DeviceScene(s) for s, _ in scenes_frames]
    pipe = P.TiledGaussianPipeline(dss[0].data(), pipeline_options(scenes_frames[0][1], precision, capacity))
    if tuning:
        pipe.set_tuning(tuning)
    targets, views = [], []
    for ds, (scene, frame) in zip(dss, scenes_frames):
        W, H = int(frame["width"]), int(frame["height"])
        dtype = torch.float16 if color_format == "rgba16f" else torch.float32
        color = torch.zeros((H, W, 4), dtype=dtype, device="cuda")
        depth = torch.zeros((H, W), dtype=torch.float32, device="cuda")
        targets.append((color, depth))
        views.append((ds.data(), P.make_camera(frame), W, H, color.data_ptr(), depth.data_ptr(), color_format))
    pipe.render_batch(views)
    stats = pipe.read_stats()
    r = pipe.get_resources()
    item_base, tile_base = pipe.batch_layout()
    vis = dev.to_numpy(r.visible_state, (4,))
    state = dev.to_numpy(r.dispatch_state, (4,))
    V, cnt = int(vis[0]), int(state[0])
    total_items, total_tiles = item_base[-1], tile_base[-1]
    g = {
        "proj_mean": dev.to_numpy(r.projected_mean, (total_items, 4), np.float32),
        "proj_conic": dev.to_numpy(r.projected_conic, (total_items, 4), np.float32),
        "proj_color": dev.to_numpy(r.projected_color, (total_items, 4), np.float32),
        "tile_counts": dev.to_numpy(r.tile_counts, (total_items,)),
        "visible_offsets": dev.to_numpy(r.visible_offsets, (total_items,)),
        "depth_keys": dev.to_numpy(r.depth_sorted_keys, (V,)),
        "depth_ids": dev.to_numpy(r.depth_sorted_ids, (V,)),
        "ordered_counts": dev.to_numpy(r.depth_ordered_tile_counts, (V,)),
        "tiles": dev.to_numpy(r.sorted_tile_ids, (cnt,)),
        "gids": dev.to_numpy(r.sorted_gaussian_ids, (cnt,)),
        "tile_offsets": dev.to_numpy(r.tile_offsets, (total_tiles + 1,)),
    }
    out = []
    for i, (ds, (scene, frame)) in enumerate(zip(dss, scenes_frames)):
        a, n = item_base[i], ds.active_count
        t0, t1 = tile_base[i], tile_base[i + 1]
        sel = (g["depth_ids"] >= a) & (g["depth_ids"] < a + n)
        lo, hi = int(g["tile_offsets"][t0]), int(g["tile_offsets"][t1])
        color, depth = targets[i]
        out.append({
            "proj_mean": g["proj_mean"][a:a + n], "proj_conic": g["proj_conic"][a:a + n],
            "proj_color": g["proj_color"][a:a + n], "tile_counts": g["tile_counts"][a:a + n],
            "visible_offsets": g["visible_offsets"][a:a + n] - g["visible_offsets"][a] if n else g["visible_offsets"][:0],
            "depth_sorted": np.stack([g["depth_keys"][sel], g["depth_ids"][sel] - a], 1),
            "ordered_counts": g["ordered_counts"][sel],
            "sorted_records": np.stack([g["tiles"][lo:hi] - t0, g["gids"][lo:hi] - a], 1),
            "tile_offsets": g["tile_offsets"][t0:t1 + 1] - lo,
            "rgba": color.float().cpu().numpy(), "depth": depth.cpu().numpy(),
        })
    pipe.dispose()
    return out, stats
