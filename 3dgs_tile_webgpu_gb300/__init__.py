"""GB300-native tiled Gaussian-splatting pass behind a C ABI.

The CUDA library (``csrc/``, built into ``_build/libgs3d.so`` by ``build.py``)
replaces the data path of the reference's ``TiledGaussianPipeline``
(src/renderer/pipeline/TiledGaussianPipeline.ts:39-484). This module is the
host-side mirror of that class for Python callers and tests: the same method
names, argument meaning and error behaviour (``RangeError``/``TypeError``/
``Error`` become ``ValueError``/``TypeError``/``RuntimeError``), calling the C
ABI through ctypes. Device memory, when the caller has none of its own, comes
from torch; torch is plumbing only, every kernel is in the library.

There is no CPU fallback: if the library cannot be loaded every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import abi
from .abi import (GS3D_OK, Camera, GaussianData, PipelineDesc, ProfileStats, Resources, SplatSource, Stats,
                  Targets, Tuning, View)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgs3d.so")
_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _LIB_PATH


def load(build_if_missing: bool = True):
    """Load libgs3d.so (building it first when absent or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing:
                from . import build as _build
                _build.build()
            if not os.path.exists(_LIB_PATH):
                raise RuntimeError(f"CUDA library missing: {_LIB_PATH} (run build.py)")
            _lib = abi.bind(C.CDLL(_LIB_PATH))
    return _lib


class GaussianPassError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _raise(lib, status: int, pipeline=None, context: str = "") -> None:
    if status == GS3D_OK:
        return
    msg = lib.gs3d_pipeline_last_error(pipeline).decode() if pipeline else ""
    msg = msg or lib.gs3d_status_string(status).decode()
    if context:
        msg = f"{context}: {msg}"
    if status == abi.GS3D_ERROR_RANGE:
        raise ValueError(msg)
    if status == abi.GS3D_ERROR_INVALID_ARGUMENT:
        raise TypeError(msg)
    raise GaussianPassError(status, msg)


def gaussian_data_from_tensors(count: int, active_count: int, sh_degree: int, means, scales_opacity,
                               rotations, sh_coefficients) -> GaussianData:
    """Describe resident device buffers (torch tensors or raw pointers) as GaussianData."""
    def ptr(x):
        return int(x.data_ptr()) if hasattr(x, "data_ptr") else int(x)
    d = GaussianData()
    d.count, d.active_count, d.sh_degree = int(count), int(active_count), int(sh_degree)
    d.means, d.scales_opacity = ptr(means), ptr(scales_opacity)
    d.rotations, d.sh_coefficients = ptr(rotations), ptr(sh_coefficients)
    return d


def default_options() -> dict:
    """The reference's pass defaults (GaussianPass.ts:170-256)."""
    return {
        "depth_sort_mode": "float32", "antialias_mode": "compensated",
        "intersection_capacity": 262_144, "background": (0.0, 0.0, 0.0, 0.0),
        "max_rasterized_splats_per_tile": None, "raster_chunk_size": 8192,
        "subpixel_sample_culling": True, "raster_transmittance_threshold": 1e-4,
        "depth_alpha_threshold": 0.95, "filter_variance": 0.3, "invalid_depth_value": 1.0,
        "boundary_policy": "clip", "raster_precision": "fp32", "depth_encoding": "device",
        "raster_stats": False, "projection_precision": "fp32", "device": 0,
    }


def make_desc(options: dict | None = None) -> PipelineDesc:
    lib = load()
    o = default_options()
    o.update(options or {})
    d = PipelineDesc()
    lib.gs3d_pipeline_desc_defaults(C.byref(d))
    d.device = int(o["device"])
    d.depth_sort_mode = {"float32": 0, "packed16": 1}[o["depth_sort_mode"]]
    d.antialias_mode = {"compensated": 0, "classic": 1}[o["antialias_mode"]]
    d.intersection_capacity = int(o["intersection_capacity"])
    d.background[:] = [float(v) for v in o["background"]]
    d.max_rasterized_splats_per_tile = int(o["max_rasterized_splats_per_tile"] or 0)
    d.raster_chunk_size = int(o["raster_chunk_size"] or 0)
    d.subpixel_sample_culling = 1 if o["subpixel_sample_culling"] else 0
    d.raster_transmittance_threshold = float(o["raster_transmittance_threshold"])
    d.depth_alpha_threshold = float(o["depth_alpha_threshold"])
    d.filter_variance = float(o["filter_variance"])
    d.invalid_depth_value = float(o["invalid_depth_value"])
    d.boundary_policy = {"clip": 0, "repeat-x": 1, "repeat-y": 2}[o["boundary_policy"]]
    d.raster_precision = {"fp32": 0, "exact": 1, "half2": 2}[o["raster_precision"]]
    d.depth_encoding = {"device": 0, "raw": 1}[o["depth_encoding"]]
    d.raster_stats = 1 if o["raster_stats"] else 0
    d.projection_precision = {"fp32": 0, "fp64": 1}[o["projection_precision"]]
    return d


def make_camera(frame: dict) -> Camera:
    """gs3d_camera from a frame dict (see ``scenes.make_frame``)."""
    import numpy as np
    cam = Camera()
    cam.projection[:] = [float(v) for v in np.asarray(frame["projection"], np.float32).ravel()]
    view = frame.get("view")
    if view is not None:
        cam.view[:] = [float(v) for v in np.asarray(view, np.float32).ravel()]
    cam.depth_near = float(frame["near"])
    cam.depth_far = float(frame["far"])
    table = np.ascontiguousarray(frame["objects"], np.float32)
    cam._table = table
    cam.object_table = table.ctypes.data_as(C.POINTER(C.c_float))
    cam.object_count = table.size // 40
    return cam


class TiledGaussianPipeline:
    """Mirror of the reference's TiledGaussianPipeline over the C ABI.

    ``data`` is a :class:`GaussianData` describing resident device buffers.
    Lifecycle: ``prepare_frame(width, height)`` then ``render(camera, ...)``
    any number of times; ``update_data``, ``resize_intersections``,
    ``read_stats``, ``get_resources``, ``dispose``.
    """

    def __init__(self, data: GaussianData, options: dict | None = None):
        self._lib = load()
        self._p = C.c_void_p()
        self._desc = make_desc(options)
        self._data = data
        st = self._lib.gs3d_pipeline_create(C.byref(self._desc), C.byref(data), C.byref(self._p))
        if st != GS3D_OK:
            _raise(self._lib, st, None, "TiledGaussianPipeline")
        self.width = self.height = 0

    # -- reference surface -------------------------------------------------
    def update_data(self, data: GaussianData) -> None:
        _raise(self._lib, self._lib.gs3d_pipeline_update_data(self._p, C.byref(data)), self._p)
        self._data = data

    def resize_intersections(self, capacity: int) -> None:
        _raise(self._lib, self._lib.gs3d_pipeline_resize_intersections(self._p, int(capacity)), self._p)

    def prepare_frame(self, width: int, height: int) -> None:
        _raise(self._lib, self._lib.gs3d_pipeline_prepare_frame(self._p, int(width), int(height)), self._p)
        self.width, self.height = int(width), int(height)

    def render(self, camera: Camera, color_ptr: int, depth_ptr: int = 0, attempt: int = 1,
               reset_valid: bool = False, color_format: str = "rgba32f", stream: int = 0) -> None:
        t = Targets()
        t.color = int(color_ptr)
        t.color_format = {"rgba16f": 0, "rgba32f": 1}[color_format]
        t.depth = C.cast(C.c_void_p(int(depth_ptr)), C.POINTER(C.c_float)) if depth_ptr else None
        st = self._lib.gs3d_pipeline_render(self._p, C.byref(camera), int(attempt), 1 if reset_valid else 0,
                                            C.byref(t), C.c_void_p(int(stream)))
        _raise(self._lib, st, self._p)

    def render_batch(self, views: list, attempt: int = 1, reset_valid: bool = False, stream: int = 0) -> None:
        """Render several views in one launch sequence.

        ``views`` holds (GaussianData, Camera, width, height, color_ptr,
        depth_ptr, color_format) tuples."""
        arr = (View * len(views))()
        keep = []
        for i, (data, cam, w, h, color_ptr, depth_ptr, fmt) in enumerate(views):
            arr[i].data = C.pointer(data)
            arr[i].camera = C.pointer(cam)
            arr[i].width, arr[i].height = int(w), int(h)
            arr[i].targets.color = int(color_ptr)
            arr[i].targets.color_format = {"rgba16f": 0, "rgba32f": 1}[fmt]
            arr[i].targets.depth = (C.cast(C.c_void_p(int(depth_ptr)), C.POINTER(C.c_float))
                                    if depth_ptr else None)
            keep.append((data, cam))
        st = self._lib.gs3d_pipeline_render_batch(self._p, arr, len(views), int(attempt), 1 if reset_valid else 0,
                                                  C.c_void_p(int(stream)))
        _raise(self._lib, st, self._p)

    def _views_array(self, views: list):
        arr = (View * len(views))()
        keep = []
        for i, (data, cam, w, h, color_ptr, depth_ptr, fmt) in enumerate(views):
            arr[i].data = C.pointer(data)
            arr[i].camera = C.pointer(cam)
            arr[i].width, arr[i].height = int(w), int(h)
            arr[i].targets.color = int(color_ptr)
            arr[i].targets.color_format = {"rgba16f": 0, "rgba32f": 1}[fmt]
            arr[i].targets.depth = (C.cast(C.c_void_p(int(depth_ptr)), C.POINTER(C.c_float))
                                    if depth_ptr else None)
            keep.append((data, cam))
        return arr, keep

    def set_tuning(self, tuning: dict) -> None:
        """Launch shape: ``views_per_launch`` (0 = a whole batch at once),
        ``tile_digit_bits`` (4..8), ``work_order`` (1 = heaviest tiles first)
        change nothing the batch produces; ``tile_size`` (8, 16 or 32; 0 =
        16) sets the tiles of batched renders, which leaves the EXACT image
        unchanged but not the per-tile buffers; ``raster_pixels_per_lane``
        (2 or 4) sets the fast rasterizers' block shape."""
        t = Tuning()
        self._lib.gs3d_pipeline_get_tuning(self._p, C.byref(t))
        for k, v in tuning.items():
            setattr(t, k, int(v))
        _raise(self._lib, self._lib.gs3d_pipeline_set_tuning(self._p, C.byref(t)), self._p)

    def get_tuning(self) -> dict:
        t = Tuning()
        _raise(self._lib, self._lib.gs3d_pipeline_get_tuning(self._p, C.byref(t)), self._p)
        return {"views_per_launch": t.views_per_launch, "tile_digit_bits": t.tile_digit_bits,
                "work_order": t.work_order, "tile_size": t.tile_size or 16,
                "raster_pixels_per_lane": t.raster_pixels_per_lane or 2}

    def autotune(self, views: list, trials: int = 3, stream: int = 0) -> tuple[dict, float]:
        """Time candidate tunings on this batch (same tuple layout as
        render_batch), keep the fastest; returns (tuning, ms per batch)."""
        arr, keep = self._views_array(views)
        t, ms = Tuning(), C.c_double()
        _raise(self._lib, self._lib.gs3d_pipeline_autotune(self._p, arr, len(views), int(trials), C.byref(t),
                                                           C.byref(ms), C.c_void_p(int(stream))), self._p)
        del keep
        return self.get_tuning(), float(ms.value)

    def capture_graph(self, views: list, stream: int) -> None:
        """Capture the batched pass for these views into CUDA graphs (same
        tuple layout as render_batch); launch_graph replays it with new
        cameras. ``stream`` must be a non-default CUDA stream handle."""
        arr, keep = self._views_array(views)
        self._graph_keep = (arr, keep)  # the library keeps pointers to the GaussianData structs
        _raise(self._lib, self._lib.gs3d_pipeline_capture_graph(self._p, arr, len(views), C.c_void_p(int(stream))),
               self._p)

    def launch_graph(self, cameras: list, attempt: int = 1, reset_valid: bool = False, stream: int = 0) -> None:
        arr = (Camera * len(cameras))(*cameras)
        self._graph_cams = (arr, [getattr(c, "_table", None) for c in cameras])
        st = self._lib.gs3d_pipeline_launch_graph(self._p, arr, len(cameras), int(attempt), 1 if reset_valid else 0,
                                                  C.c_void_p(int(stream)))
        _raise(self._lib, st, self._p)

    def batch_layout(self) -> tuple[list, list]:
        """(item_base, tile_base) of the last render, one entry per view plus the total."""
        n = C.c_uint32()
        self._lib.gs3d_pipeline_batch_layout(self._p, None, None, 0, C.byref(n))
        items = (C.c_uint32 * (n.value + 1))()
        tiles = (C.c_uint32 * (n.value + 1))()
        _raise(self._lib, self._lib.gs3d_pipeline_batch_layout(self._p, items, tiles, n.value + 1, C.byref(n)),
               self._p)
        return list(items), list(tiles)

    @staticmethod
    def _stats_dict(s: Stats) -> dict:
        return {"visibleGaussianCount": s.visible_gaussian_count, "intersectionCount": s.intersection_count,
                "requestedIntersections": s.requested_intersections,
                "intersectionCapacity": int(s.intersection_capacity), "overflow": bool(s.overflow),
                "deviceError": int(s.device_error),
                "rasterWork": {"checked": int(s.raster_checked), "blended": int(s.raster_blended),
                               "pixels": int(s.raster_pixels), "alphaStopped": int(s.raster_alpha_stopped)},
                "outputState": [int(v) for v in s.output_state]}

    def read_stats(self) -> dict:
        s = Stats()
        st = self._lib.gs3d_pipeline_read_stats(self._p, C.byref(s))
        out = self._stats_dict(s)
        _raise(self._lib, st, self._p)
        return out

    def request_stats(self, stream: int = 0) -> None:
        """Enqueue the asynchronous read-back of the last render's counters
        (one in flight per pipeline); ``poll_stats`` collects it."""
        _raise(self._lib, self._lib.gs3d_pipeline_request_stats(self._p, C.c_void_p(int(stream))), self._p)

    def poll_stats(self, wait: bool = False):
        """The requested counters as read_stats returns them, or None while the
        copy is still in flight (``wait`` blocks until it lands)."""
        s = Stats()
        st = self._lib.gs3d_pipeline_poll_stats(self._p, C.byref(s), 1 if wait else 0)
        if st == abi.GS3D_NOT_READY:
            return None
        out = self._stats_dict(s)
        _raise(self._lib, st, self._p)
        return out

    def set_wait_limit(self, polls: int) -> None:
        """Polls a look-back wait may spend on one status word before the
        frame reports a device timeout (0: the default, about one second)."""
        _raise(self._lib, self._lib.gs3d_pipeline_set_wait_limit(self._p, int(polls)), self._p)

    def debug_withhold_chunk(self) -> None:
        """Test hook: the next render's compaction never scans its first
        chunk, so the next chunk's look-back wait runs out."""
        _raise(self._lib, self._lib.gs3d_pipeline_debug_withhold_chunk(self._p), self._p)

    def read_profile(self) -> dict:
        """GaussianPassProfileStats of the last render (types.ts:105-148):
        tileLoads, appliedTileCap (None without maxRasterizedSplatsPerTile),
        tileCapEstimates at 2048/4096/8192, zeroPixelSubpixelSplats."""
        s = ProfileStats()
        _raise(self._lib, self._lib.gs3d_pipeline_read_profile(self._p, C.byref(s)), self._p)
        L = s.tile_loads

        def cap(c):
            return {"cap": c.cap, "rasterizedIntersections": c.rasterized_intersections,
                    "droppedIntersections": c.dropped_intersections, "droppedFraction": c.dropped_fraction,
                    "affectedTiles": c.affected_tiles, "totalBatches": c.total_batches, "maxBatches": c.max_batches}

        return {
            "tileLoads": {"max": L.max, "mean": L.mean, "median": L.median, "p95": L.p95, "p99": L.p99,
                          "tilesOver256": L.tiles_over_256, "tilesOver512": L.tiles_over_512,
                          "tilesOver1024": L.tiles_over_1024, "tilesOver2048": L.tiles_over_2048,
                          "totalBatches": L.total_batches, "maxBatches": L.max_batches},
            "appliedTileCap": cap(s.applied_cap) if s.has_applied_cap else None,
            "tileCapEstimates": [cap(c) for c in s.cap_estimates],
            "zeroPixelSubpixelSplats": s.zero_pixel_subpixel_splats,
        }

    def get_resources(self) -> Resources:
        r = Resources()
        _raise(self._lib, self._lib.gs3d_pipeline_get_resources(self._p, C.byref(r)), self._p)
        return r

    def set_profiling(self, enabled: bool) -> None:
        _raise(self._lib, self._lib.gs3d_pipeline_set_profiling(self._p, 1 if enabled else 0), self._p)

    def stage_times(self) -> tuple[dict, int]:
        """Mean per-stage milliseconds over the renders profiled since the last call."""
        ms = (C.c_float * len(abi.STAGES))()
        n = C.c_uint32()
        _raise(self._lib, self._lib.gs3d_pipeline_stage_times(self._p, ms, C.byref(n)), self._p)
        return {name: float(ms[i]) for i, name in enumerate(abi.STAGES)}, int(n.value)

    def last_launch_count(self) -> int:
        return int(self._lib.gs3d_pipeline_last_launch_count(self._p))

    def dispose(self) -> None:
        if self._p:
            self._lib.gs3d_pipeline_destroy(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.dispose()
        except Exception:
            pass


def debug_fail_allocation(nth: int) -> None:
    """Test hook: the nth device allocation the library makes from now on
    (1 = the next one) fails as out of memory; 0 disarms."""
    load().gs3d_debug_fail_allocation(int(nth))


def pack_splats(centers, scales, opacity, quaternions, rgb, sh_rest, first_slot: int, means, scales_opacity,
                rotations, sh_coefficients, capacity: int, object_id: int = 0, stream: int = 0) -> None:
    """Encode linear splat attributes into slots [first_slot, first_slot + n)
    of a store's packed device buffers on the GPU (the compact layout of the
    reference's Rust packer, engine.rs:1801-1891). Arguments are CUDA tensors:
    centers/scales (n, 3), opacity (n,), quaternions (n, 4) xyzw, rgb (n, 3),
    sh_rest (n, C-1, 3) or None; outputs as in ``scenes.pack_scene``."""
    lib = load()
    n = int(centers.shape[0])
    degree = 0 if sh_rest is None else int(round((int(sh_rest.shape[1]) + 1) ** 0.5)) - 1
    src = SplatSource()
    src.centers, src.scales, src.opacity = centers.data_ptr(), scales.data_ptr(), opacity.data_ptr()
    src.quaternions, src.rgb = quaternions.data_ptr(), rgb.data_ptr()
    src.sh_rest = sh_rest.data_ptr() if sh_rest is not None else None
    src.count, src.sh_degree, src.object_id = n, degree, int(object_id)
    _raise(lib, lib.gs3d_pack_splats(C.byref(src), int(first_slot), means.data_ptr(), scales_opacity.data_ptr(),
                                     rotations.data_ptr(), sh_coefficients.data_ptr(), int(capacity),
                                     C.c_void_p(int(stream))))
