"""CPU oracle for the tiled Gaussian-splatting pass (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; it is the checker, never the product path.
It wraps ``gs_oracle.cpp`` (a restatement of the reference's WGSL/TSL
kernels, see that file's header for the reference file:line map) through
ctypes.

Parity status: function-level pins come from the reference's executed-WGSL
known-answer tests (ported in tests/test_oracle_known_answers.py); the
reference ships no rendered-image golden, so image-level parity is pinned
only through those function-level tests.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libgs_oracle.so")
_SRC = [os.path.join(_HERE, "gs_oracle.cpp"),
        os.path.join(_HERE, "..", "3dgs_tile_webgpu_gb300", "csrc", "detmath.h")]
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no FMA contraction, OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _SRC)
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= newest:
        return _SO
    tmp = _SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-o", tmp, _SRC[0]]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


class GsoScene(C.Structure):
    _fields_ = [("count", C.c_uint32), ("active_count", C.c_uint32),
                ("sh_degree", C.c_uint32), ("_pad", C.c_uint32),
                ("means", C.c_void_p), ("shape", C.c_void_p),
                ("rotations", C.c_void_p), ("sh", C.c_void_p)]


class GsoFrame(C.Structure):
    _fields_ = [("projection", C.c_float * 16), ("viewport", C.c_float * 4),
                ("filter_variance", C.c_float), ("boundary_axis", C.c_uint32),
                ("object_count", C.c_uint32), ("depth_sort_mode", C.c_uint32),
                ("objects", C.c_void_p), ("background", C.c_float * 4),
                ("transmittance_threshold", C.c_float),
                ("depth_alpha_threshold", C.c_float),
                ("invalid_depth_value", C.c_float), ("antialias", C.c_uint32),
                ("subpixel_culling", C.c_uint32), ("raster_chunk_size", C.c_uint32),
                ("max_splats_per_tile", C.c_uint32), ("capacity", C.c_uint32),
                ("depth_encoding", C.c_uint32), ("attempt", C.c_uint32),
                ("last_version", C.c_uint32), ("reset_valid", C.c_uint32),
                ("_pad", C.c_uint32)]


class GsoOutputs(C.Structure):
    _fields_ = [("proj_mean", C.c_void_p), ("proj_conic", C.c_void_p),
                ("proj_color", C.c_void_p), ("tile_counts", C.c_void_p),
                ("visible_offsets", C.c_void_p), ("depth_sorted", C.c_void_p),
                ("ordered_counts", C.c_void_p), ("intersection_offsets", C.c_void_p),
                ("visible_state", C.c_uint32 * 4), ("state", C.c_uint32 * 4),
                ("output_state", C.c_uint32 * 4), ("sorted_records", C.c_void_p),
                ("tile_offsets", C.c_void_p), ("rgba", C.c_void_p),
                ("depth", C.c_void_p), ("checked", C.c_uint64),
                ("blended", C.c_uint64)]


_F = C.c_float
_FP = C.POINTER(C.c_float)
_U = C.c_uint32


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            for name in ("gso_expf", "gso_logf", "gso_sinf", "gso_cosf"):
                getattr(L, name).restype = _F
                getattr(L, name).argtypes = [_F]
            L.gso_atan2f.restype = _F
            L.gso_atan2f.argtypes = [_F, _F]
            L.gso_half_to_float.restype = _F
            L.gso_half_to_float.argtypes = [_U]
            L.gso_decode_scale_opacity.argtypes = [_U, _U, _FP]
            L.gso_decode_rotation.argtypes = [_U, _FP]
            L.gso_decode_sh.argtypes = [_U, _FP]
            L.gso_pack_sh.restype = _U
            L.gso_pack_sh.argtypes = [_FP]
            L.gso_encode_oct101012.restype = _U
            L.gso_encode_oct101012.argtypes = [_FP]
            L.gso_zero_pixel_flag.restype = _U
            L.gso_zero_pixel_flag.argtypes = [_FP, _FP, _U, _U]
            L.gso_f16_bits.restype = _U
            L.gso_f16_bits.argtypes = [_F]
            L.gso_pack_splat.restype = None
            L.gso_pack_splat.argtypes = [_FP, _FP, _F, _FP, _FP, _FP, _U, _U, _FP, C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
            L.gso_view_covariance.argtypes = [_FP, _FP, _FP, _FP]
            L.gso_projection_result.argtypes = [_FP, _F, _FP, _F, _FP]
            L.gso_perspective_projection.argtypes = [_FP, _FP, _FP, _FP, _F, _FP]
            L.gso_projection_is_valid.restype = C.c_int
            L.gso_projection_is_valid.argtypes = [_FP]
            L.gso_boundary_delta.argtypes = [_FP, _FP, _FP, _FP, _U, _FP]
            L.gso_boundary_tile_hit.restype = C.c_int
            L.gso_boundary_tile_hit.argtypes = [_FP, _FP, _F, _FP, C.c_int, C.c_int, _FP, _U]
            L.gso_count_tiles.restype = _U
            L.gso_count_tiles.argtypes = [_FP, _FP, _F, _FP, C.c_int, C.c_int, C.c_int,
                                          C.c_int, _FP, _U]
            L.gso_subpixel_has_sample.restype = C.c_int
            L.gso_subpixel_has_sample.argtypes = [_FP, _FP, _F, _FP, _U, _U, _U]
            L.gso_finalize_depth.restype = _F
            L.gso_finalize_depth.argtypes = [_F, _F, _F, _F, _F, _F, C.c_int]
            L.gso_tile_sort_bits.restype = _U
            L.gso_tile_sort_bits.argtypes = [_U]
            L.gso_num_threads.restype = C.c_int
            L.gso_render.restype = C.c_int
            L.gso_render.argtypes = [C.POINTER(GsoScene), C.POINTER(GsoFrame),
                                     C.POINTER(GsoOutputs), C.c_int]
            _lib = L
    return _lib


def f32(values) -> "C.Array":
    a = np.ascontiguousarray(np.asarray(values, dtype=np.float32).ravel())
    return (C.c_float * a.size)(*a.tolist())


def out_f32(n: int):
    return (C.c_float * n)()


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None else 0


def make_frame(frame: dict) -> GsoFrame:
    """Translate a frame dict (see the package's frame helpers) into GsoFrame."""
    fr = GsoFrame()
    fr.projection[:] = [float(v) for v in np.asarray(frame["projection"], np.float32).ravel()]
    fr.viewport[:] = [float(frame["width"]), float(frame["height"]),
                      float(frame["near"]), float(frame["far"])]
    fr.filter_variance = float(frame.get("filter_variance", 0.3))
    fr.boundary_axis = int(frame.get("boundary_axis", 0))
    objects = np.ascontiguousarray(frame["objects"], dtype=np.float32)
    fr.object_count = objects.size // 40
    fr.objects = objects.ctypes.data
    fr.depth_sort_mode = int(frame.get("depth_sort_mode", 0))
    fr.background[:] = [float(v) for v in frame.get("background", (0, 0, 0, 0))]
    fr.transmittance_threshold = float(frame.get("transmittance_threshold", 1e-4))
    fr.depth_alpha_threshold = float(frame.get("depth_alpha_threshold", 0.95))
    fr.invalid_depth_value = float(frame.get("invalid_depth_value", 1.0))
    fr.antialias = int(frame.get("antialias", 0))
    fr.subpixel_culling = int(frame.get("subpixel_culling", 1))
    fr.raster_chunk_size = int(frame.get("raster_chunk_size", 8192))
    fr.max_splats_per_tile = int(frame.get("max_splats_per_tile", 0))
    fr.capacity = int(frame.get("capacity", 0xFFFFFFFF))
    fr.depth_encoding = int(frame.get("depth_encoding", 0))
    fr.attempt = int(frame.get("attempt", 1))
    fr.last_version = int(frame.get("last_version", 0))
    fr.reset_valid = int(frame.get("reset_valid", 0))
    fr._keep = objects  # keep the table alive with the struct
    return fr


def render(scene: dict, frame: dict, precision: int = 0, output_depth: bool = True,
           rgba_init: np.ndarray | None = None) -> dict:
    """Run the whole pass on the CPU. precision 0 = FP32 restatement, 1 = FP64 twin.

    Returns every intermediate buffer the reference exposes through
    ``TiledGaussianPipeline.getResources()`` plus the image.
    """
    L = lib()
    n = int(scene["active_count"])
    count = int(scene["count"])
    sc = GsoScene()
    sc.count = count
    sc.active_count = n
    sc.sh_degree = int(scene["sh_degree"])
    means = np.ascontiguousarray(scene["means"], np.float32)
    shape = np.ascontiguousarray(scene["shape"], np.uint32)
    rot = np.ascontiguousarray(scene["rotations"], np.uint32)
    sh = np.ascontiguousarray(scene["sh"], np.uint32)
    sc.means, sc.shape, sc.rotations, sc.sh = (_ptr(means), _ptr(shape), _ptr(rot), _ptr(sh))
    fr = make_frame(frame)
    W, H = int(frame["width"]), int(frame["height"])
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    capacity_alloc = int(frame.get("capacity_alloc", 0)) or None
    res = {
        "proj_mean": np.zeros((n, 4), np.float32),
        "proj_conic": np.zeros((n, 4), np.float32),
        "proj_color": np.zeros((n, 4), np.float32),
        "tile_counts": np.zeros(n, np.uint32),
        "visible_offsets": np.zeros(n, np.uint32),
        "depth_sorted": np.zeros((max(n, 1), 2), np.uint32),
        "ordered_counts": np.zeros(max(n, 1), np.uint32),
        "intersection_offsets": np.zeros(max(n, 1), np.uint32),
        "tile_offsets": np.zeros(tiles + 1, np.uint32),
        "rgba": (np.zeros((H, W, 4), np.float32) if rgba_init is None
                 else np.ascontiguousarray(rgba_init, np.float32).copy()),
        "depth": np.zeros((H, W), np.float32) if output_depth else None,
    }
    # The record buffer must hold every emitted record: size it from a count
    # pass when no explicit allocation is given.
    if capacity_alloc is None:
        est = _estimate_records(L, sc, fr, n)
        # The FP64 twin may count a few borderline tiles differently.
        capacity_alloc = est if precision == 0 else est + est // 50 + 4096
    # Never let the oracle write past the record buffer it was given.
    fr.capacity = min(int(fr.capacity), int(capacity_alloc))
    res["sorted_records"] = np.zeros((max(capacity_alloc, 1), 2), np.uint32)
    out = GsoOutputs()
    for k in ("proj_mean", "proj_conic", "proj_color", "tile_counts", "visible_offsets",
              "depth_sorted", "ordered_counts", "intersection_offsets", "sorted_records",
              "tile_offsets", "rgba", "depth"):
        setattr(out, k, _ptr(res[k]))
    L.gso_render(C.byref(sc), C.byref(fr), C.byref(out), int(precision))
    res["visible_state"] = np.array(out.visible_state[:], np.uint32)
    res["state"] = np.array(out.state[:], np.uint32)
    res["output_state"] = np.array(out.output_state[:], np.uint32)
    res["checked"] = int(out.checked)
    res["blended"] = int(out.blended)
    V = int(res["visible_state"][0])
    cnt = int(res["state"][0])
    res["depth_sorted"] = res["depth_sorted"][:V]
    res["ordered_counts"] = res["ordered_counts"][:V]
    res["intersection_offsets"] = res["intersection_offsets"][:V]
    res["sorted_records"] = res["sorted_records"][:cnt]
    res["tiles_x"] = (W + 15) // 16
    res["tiles_y"] = (H + 15) // 16
    return res


def _estimate_records(L, sc, fr, n) -> int:
    """Total intersections of this frame (a counting pass).

    Capacity 0 makes any non-empty frame overflow, which skips emission and
    raster; an empty frame still rasterizes (background only), so every
    buffer here is sized for the full frame and kept alive for the call."""
    probe = GsoFrame.from_buffer_copy(fr)
    probe.capacity = 0
    W, H = int(fr.viewport[0]), int(fr.viewport[1])
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    m = max(n, 1)
    keep = {
        "m": np.zeros(m * 4, np.float32), "c": np.zeros(m * 4, np.float32), "col": np.zeros(m * 4, np.float32),
        "tc": np.zeros(m, np.uint32), "vo": np.zeros(m, np.uint32), "oc": np.zeros(m, np.uint32),
        "io": np.zeros(m, np.uint32), "ds": np.zeros(m * 2, np.uint32), "to": np.zeros(tiles + 1, np.uint32),
        "rg": np.zeros(W * H * 4, np.float32), "sr": np.zeros(2, np.uint32),
    }
    out = GsoOutputs()
    out.proj_mean, out.proj_conic, out.proj_color = _ptr(keep["m"]), _ptr(keep["c"]), _ptr(keep["col"])
    out.tile_counts, out.visible_offsets = _ptr(keep["tc"]), _ptr(keep["vo"])
    out.ordered_counts, out.intersection_offsets = _ptr(keep["oc"]), _ptr(keep["io"])
    out.depth_sorted, out.tile_offsets, out.rgba, out.depth = _ptr(keep["ds"]), _ptr(keep["to"]), _ptr(keep["rg"]), 0
    out.sorted_records = _ptr(keep["sr"])
    L.gso_render(C.byref(sc), C.byref(probe), C.byref(out), 0)
    return int(out.state[1])


def pack_splats(centers, scales, opacity, quats, rgb, sh_rest, object_id: int = 0) -> dict:
    """The compact packed buffers of linear splat attributes, one splat at a
    time through the C restatement of the reference's CPU packer (libm, like
    the Rust backend): checks the on-device packer."""
    L = lib()
    n = int(np.asarray(centers).shape[0])
    C_ = 1 + (0 if sh_rest is None else int(np.asarray(sh_rest).shape[1]))
    centers = np.ascontiguousarray(centers, np.float32)
    scales = np.ascontiguousarray(scales, np.float32)
    opacity = np.ascontiguousarray(opacity, np.float32)
    quats = np.ascontiguousarray(quats, np.float32)
    rgb = np.ascontiguousarray(rgb, np.float32)
    rest = np.ascontiguousarray(sh_rest if sh_rest is not None else np.zeros((n, 0, 3)), np.float32)
    means = np.zeros((n, 4), np.float32)
    shape = np.zeros((n, 2), np.uint32)
    rot = np.zeros(n, np.uint32)
    sh = np.zeros((n, C_), np.uint32)
    fp = C.POINTER(C.c_float)
    up = C.POINTER(C.c_uint32)
    for i in range(n):
        L.gso_pack_splat(centers[i].ctypes.data_as(fp), scales[i].ctypes.data_as(fp), float(opacity[i]),
                         quats[i].ctypes.data_as(fp), rgb[i].ctypes.data_as(fp), rest[i].ctypes.data_as(fp), C_,
                         int(object_id), means[i].ctypes.data_as(fp), shape[i].ctypes.data_as(up),
                         rot[i:i + 1].ctypes.data_as(up), sh[i].ctypes.data_as(up))
    return {"means": means, "shape": shape, "rotations": rot, "sh": sh}
