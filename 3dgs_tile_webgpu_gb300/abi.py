"""ctypes mirror of include/gs3d.h (structures, enums and function signatures)."""
from __future__ import annotations

import ctypes as C

GS3D_ABI_VERSION = 4
GS3D_OK = 0
GS3D_ERROR_INVALID_ARGUMENT = 1
GS3D_ERROR_RANGE = 2
GS3D_ERROR_NOT_PREPARED = 3
GS3D_ERROR_OUT_OF_MEMORY = 4
GS3D_ERROR_CUDA = 5
GS3D_ERROR_DEVICE_TIMEOUT = 6
GS3D_ERROR_UNSUPPORTED = 7
GS3D_NOT_READY = 8
STATIC_COMPACT_MAX_ITEMS = 16777216
STAGES = ("project", "compact", "depth_sort", "scan", "emit", "tile_sort", "ranges", "raster")
STATUS_NAMES = {0: "ok", 1: "invalid-argument", 2: "range", 3: "not-prepared", 4: "allocation-failed",
                5: "cuda-error", 6: "device-timeout", 7: "unsupported", 8: "not-ready"}


class GaussianData(C.Structure):
    _fields_ = [("count", C.c_uint32), ("active_count", C.c_uint32), ("sh_degree", C.c_uint32),
                ("reserved", C.c_uint32), ("means", C.c_void_p), ("scales_opacity", C.c_void_p),
                ("rotations", C.c_void_p), ("sh_coefficients", C.c_void_p)]


class PipelineDesc(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("device", C.c_int32), ("depth_sort_mode", C.c_uint32),
                ("antialias_mode", C.c_uint32), ("intersection_capacity", C.c_uint64),
                ("background", C.c_float * 4), ("max_rasterized_splats_per_tile", C.c_uint32),
                ("raster_chunk_size", C.c_uint32), ("subpixel_sample_culling", C.c_uint32),
                ("raster_transmittance_threshold", C.c_float), ("depth_alpha_threshold", C.c_float),
                ("filter_variance", C.c_float), ("invalid_depth_value", C.c_float),
                ("boundary_policy", C.c_uint32), ("raster_precision", C.c_uint32),
                ("depth_encoding", C.c_uint32), ("raster_stats", C.c_uint32),
                ("projection_precision", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("projection", C.c_float * 16), ("view", C.c_float * 16), ("depth_near", C.c_float),
                ("depth_far", C.c_float), ("object_table", C.POINTER(C.c_float)), ("object_count", C.c_uint32),
                ("reserved", C.c_uint32)]


class Targets(C.Structure):
    _fields_ = [("color", C.c_void_p), ("color_format", C.c_uint32), ("reserved", C.c_uint32),
                ("depth", C.POINTER(C.c_float))]


class View(C.Structure):
    _fields_ = [("data", C.POINTER(GaussianData)), ("camera", C.POINTER(Camera)), ("width", C.c_uint32),
                ("height", C.c_uint32), ("targets", Targets)]


class Tuning(C.Structure):
    _fields_ = [("views_per_launch", C.c_uint32), ("tile_digit_bits", C.c_uint32), ("work_order", C.c_uint32),
                ("tile_size", C.c_uint32), ("raster_pixels_per_lane", C.c_uint32), ("reserved", C.c_uint32 * 3)]


class SplatSource(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in ("centers", "scales", "opacity", "quaternions", "rgb", "sh_rest")] + \
               [("count", C.c_uint32), ("sh_degree", C.c_uint32), ("object_id", C.c_uint32), ("reserved", C.c_uint32)]


class TileLoadStats(C.Structure):
    _fields_ = [(name, C.c_uint32) for name in ("max", "p95", "p99", "tiles_over_256", "tiles_over_512",
                                                 "tiles_over_1024", "tiles_over_2048", "max_batches")] + \
               [("mean", C.c_double), ("median", C.c_double), ("total_batches", C.c_uint64)]


class TileCapStats(C.Structure):
    _fields_ = [("cap", C.c_uint32), ("affected_tiles", C.c_uint32), ("rasterized_intersections", C.c_uint64),
                ("dropped_intersections", C.c_uint64), ("dropped_fraction", C.c_double),
                ("total_batches", C.c_uint64), ("max_batches", C.c_uint32), ("reserved", C.c_uint32)]


class ProfileStats(C.Structure):
    _fields_ = [("tile_loads", TileLoadStats), ("cap_estimates", TileCapStats * 3), ("applied_cap", TileCapStats),
                ("has_applied_cap", C.c_uint32), ("zero_pixel_subpixel_splats", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("visible_gaussian_count", C.c_uint32), ("intersection_count", C.c_uint32),
                ("requested_intersections", C.c_uint32), ("overflow", C.c_uint32),
                ("intersection_capacity", C.c_uint64), ("device_error", C.c_uint32), ("reserved", C.c_uint32),
                ("raster_checked", C.c_uint64), ("raster_blended", C.c_uint64), ("raster_pixels", C.c_uint64),
                ("raster_alpha_stopped", C.c_uint64), ("output_state", C.c_uint32 * 4)]


class Resources(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "projected_mean", "projected_conic", "projected_color", "tile_counts", "visible_offsets",
        "depth_sorted_keys", "depth_sorted_ids", "depth_ordered_tile_counts", "intersection_offsets",
        "dispatch_state", "visible_state", "sorted_tile_ids", "sorted_gaussian_ids", "tile_offsets",
        "output_state")] + [("active_count", C.c_uint32), ("tiles_x", C.c_uint32), ("tiles_y", C.c_uint32),
                            ("total_tiles", C.c_uint32), ("intersection_capacity", C.c_uint64)]


# Every symbol include/gs3d.h declares, with (restype, argtypes).
_P = C.c_void_p
SIGNATURES = {
    "gs3d_abi_version": (C.c_uint32, []),
    "gs3d_status_string": (C.c_char_p, [C.c_int]),
    "gs3d_pipeline_desc_defaults": (None, [C.POINTER(PipelineDesc)]),
    "gs3d_pipeline_create": (C.c_int, [C.POINTER(PipelineDesc), C.POINTER(GaussianData), C.POINTER(C.c_void_p)]),
    "gs3d_pipeline_destroy": (None, [_P]),
    "gs3d_pipeline_update_data": (C.c_int, [_P, C.POINTER(GaussianData)]),
    "gs3d_pipeline_resize_intersections": (C.c_int, [_P, C.c_uint64]),
    "gs3d_pipeline_prepare_frame": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "gs3d_pipeline_render": (C.c_int, [_P, C.POINTER(Camera), C.c_uint32, C.c_int, C.POINTER(Targets), _P]),
    "gs3d_pipeline_render_batch": (C.c_int, [_P, C.POINTER(View), C.c_uint32, C.c_uint32, C.c_int, _P]),
    "gs3d_pipeline_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "gs3d_pipeline_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "gs3d_pipeline_autotune": (C.c_int, [_P, C.POINTER(View), C.c_uint32, C.c_uint32, C.POINTER(Tuning),
                                         C.POINTER(C.c_double), _P]),
    "gs3d_pipeline_capture_graph": (C.c_int, [_P, C.POINTER(View), C.c_uint32, _P]),
    "gs3d_pipeline_launch_graph": (C.c_int, [_P, C.POINTER(Camera), C.c_uint32, C.c_uint32, C.c_int, _P]),
    "gs3d_pipeline_batch_layout": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32,
                                             C.POINTER(C.c_uint32)]),
    "gs3d_pipeline_read_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "gs3d_pipeline_request_stats": (C.c_int, [_P, _P]),
    "gs3d_pipeline_poll_stats": (C.c_int, [_P, C.POINTER(Stats), C.c_int]),
    "gs3d_pipeline_set_wait_limit": (C.c_int, [_P, C.c_uint32]),
    "gs3d_pipeline_debug_withhold_chunk": (C.c_int, [_P]),
    "gs3d_debug_fail_allocation": (None, [C.c_uint32]),
    "gs3d_pipeline_get_resources": (C.c_int, [_P, C.POINTER(Resources)]),
    "gs3d_pipeline_read_profile": (C.c_int, [_P, C.POINTER(ProfileStats)]),
    "gs3d_pipeline_last_error": (C.c_char_p, [_P]),
    "gs3d_pipeline_last_launch_count": (C.c_uint32, [_P]),
    "gs3d_pipeline_set_profiling": (C.c_int, [_P, C.c_int]),
    "gs3d_pipeline_stage_times": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
    "gs3d_stage_name": (C.c_char_p, [C.c_uint32]),
    "gs3d_compact_visible_static": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P]),
    "gs3d_pack_splats": (C.c_int, [C.POINTER(SplatSource), C.c_uint32, _P, _P, _P, _P, C.c_uint32, _P]),
    "gs3d_capacity_next": (C.c_uint64, [C.c_uint64, C.c_double, C.c_double, C.c_uint64, C.c_uint64]),
}


def bind(lib):
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
