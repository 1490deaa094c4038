"""Packed-buffer encoders, cameras and seeded synthetic scenes.

The pass consumes the exact storage buffers the reference's Rust/WASM backend
produces (``GaussianData``, src/renderer/GaussianData.ts:10-33,108-138):

* ``means``     float32[count, 4]: local xyz, objectId (or -1 for an empty slot)
* ``shape``     uint32[count, 2]: [f16 ln sx | f16 ln sy << 16],
                [f16 ln sz | f16 opacity << 16]
                (rust/gaussian-backend/src/engine.rs:1814-1833,
                rust/vendor/spark-lib/src/splat_encode.rs:127-136)
* ``rotations`` uint32[count]: Spark oct101012 quaternion
                (rust/vendor/spark-lib/src/splat_encode.rs:234-252)
* ``sh``        uint32[count * C + count]: rgb8e8 SH coefficients
                (engine.rs:1857-1872,1940-1949) followed by the active-slot
                tail read by projection (ProjectionStage.ts:214-218,393-405)

Frames carry the column-major projection matrix (three.js
``PerspectiveCamera``), the viewport and depth range, and the per-object table
of 40 floats (matrixWorld, modelView, camera position in object space,
visibility; src/renderer/pipeline/ObjectFrameState.ts:97-119).

The synthetic generators stand in for the reference's sample scene (a git-LFS
pointer, absent here) with the distributions the benchmark configurations name.
Random numbers come from numpy's PCG64 with seed 1000 + configuration number.
"""
from __future__ import annotations

import math

import numpy as np

SH_C0 = 0.28209479177387814  # engine.rs:1858 DC normalisation


# ---------------------------------------------------------------------------
# Codecs (vectorised, float32 arithmetic like the Rust encoders).

def f16_bits(x) -> np.ndarray:
    """IEEE binary16 bits of float32 values, round to nearest even
    (Rust ``half::f16::from_f32``, half 2.7.1)."""
    return np.asarray(x, np.float32).astype(np.float16).view(np.uint16).astype(np.uint32)


def encode_oct101012(q: np.ndarray) -> np.ndarray:
    """Quaternions (N, 4) xyzw -> Spark oct101012 words.

    Follows rust/vendor/spark-lib/src/splat_encode.rs:234-252: flip to w >= 0,
    axis-angle, octahedral axis in 10+10 bits, angle/pi in 12 bits."""
    q = np.asarray(q, np.float32).reshape(-1, 4).copy()
    neg = q[:, 3] < 0
    q[neg] = -q[neg]
    with np.errstate(invalid="ignore", divide="ignore"):
        theta = (np.float32(2.0) * np.arccos(np.clip(q[:, 3], 0, 1))).astype(np.float32)
        s = np.sin(theta * np.float32(0.5)).astype(np.float32)
        small = np.abs(s) < np.float32(1e-6)
        axis = np.where(small[:, None], np.array([1, 0, 0], np.float32), q[:, :3] / s[:, None])
        axis = axis.astype(np.float32)
        ssum = (np.abs(axis[:, 0]) + np.abs(axis[:, 1]) + np.abs(axis[:, 2])).astype(np.float32)
        p = (axis[:, :2] / ssum[:, None]).astype(np.float32)
    zneg = axis[:, 2] < 0
    sgn = np.where(p >= 0, np.float32(1), np.float32(-1))
    folded = np.stack([(1 - np.abs(p[:, 1])) * sgn[:, 0], (1 - np.abs(p[:, 0])) * sgn[:, 1]], 1)
    p = np.where(zneg[:, None], folded, p).astype(np.float32)
    uv = np.clip((p * np.float32(0.5) + np.float32(0.5)) * np.float32(1023), 0, 1023)
    uv = np.floor(uv + np.float32(0.5)).astype(np.uint32)  # Rust round(): half away from zero
    r = np.clip(theta / np.float32(math.pi) * np.float32(4095), 0, 4095)
    r = np.floor(r + np.float32(0.5)).astype(np.uint32)
    return (r << 20) | (uv[:, 1] << 10) | uv[:, 0]


def pack_sh(rgb: np.ndarray) -> np.ndarray:
    """Signed RGB triples (..., 3) -> rgb8e8 words (engine.rs:1940-1949)."""
    rgb = np.asarray(rgb, np.float32)
    mx = np.max(np.abs(rgb), axis=-1)
    with np.errstate(divide="ignore"):
        e = np.clip(np.ceil(np.log2(np.where(mx > 0, mx, 1))), -126, 127).astype(np.int32)
    mult = (np.float32(127.0) / np.ldexp(np.float32(1), e).astype(np.float32)).astype(np.float32)
    b = np.clip(np.floor(rgb * mult[..., None] + np.float32(0.5)), -127, 127).astype(np.int32)
    b = b.astype(np.uint32) & 255
    word = b[..., 0] | (b[..., 1] << 8) | (b[..., 2] << 16) | ((e + 127).astype(np.uint32) << 24)
    return np.where(mx > 0, word, 0).astype(np.uint32)


def sh_coefficient_count(degree: int) -> int:
    return (degree + 1) ** 2


def pack_scene(means_xyz, object_ids, log_scales, opacity, quats, sh_rgb, active_slots=None,
               empty_slots=None) -> dict:
    """Build the packed buffers of one store layout.

    ``sh_rgb`` is (count, C, 3) with the DC term already in SH units.
    ``active_slots`` (uint32) becomes the projection's ordinal -> slot tail;
    the default draws every slot in order. ``empty_slots`` get objectId -1.
    """
    count = int(np.asarray(means_xyz).shape[0])
    C = int(np.asarray(sh_rgb).shape[1])
    degree = int(round(math.sqrt(C))) - 1
    means = np.zeros((count, 4), np.float32)
    means[:, :3] = np.asarray(means_xyz, np.float32)
    means[:, 3] = np.asarray(object_ids, np.float32)
    if empty_slots is not None:
        means[np.asarray(empty_slots), 3] = -1.0
    ls = np.asarray(log_scales, np.float32)
    op = np.asarray(opacity, np.float32)
    shape = np.zeros((count, 2), np.uint32)
    shape[:, 0] = f16_bits(ls[:, 0]) | (f16_bits(ls[:, 1]) << 16)
    shape[:, 1] = f16_bits(ls[:, 2]) | (f16_bits(op) << 16)
    rot = encode_oct101012(quats)
    if active_slots is None:
        active_slots = np.arange(count, dtype=np.uint32)
    active_slots = np.asarray(active_slots, np.uint32)
    sh = np.zeros(count * C + count, np.uint32)
    sh[: count * C] = pack_sh(sh_rgb).reshape(-1)
    sh[count * C: count * C + active_slots.size] = active_slots
    return {"count": count, "active_count": int(active_slots.size), "sh_degree": degree,
            "means": means, "shape": shape, "rotations": rot, "sh": sh}


# ---------------------------------------------------------------------------
# Cameras and frames (three.js conventions, float64 math stored as float32).

def perspective(fov_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """Column-major ``PerspectiveCamera.projectionMatrix`` (zoom 1, no film offset)."""
    top = near * math.tan(math.radians(0.5 * fov_deg))
    height = 2 * top
    width = aspect * height
    left = -0.5 * width
    right, bottom = left + width, top - height
    m = np.zeros((4, 4))
    m[0, 0] = 2 * near / (right - left)
    m[1, 1] = 2 * near / (top - bottom)
    m[0, 2] = (right + left) / (right - left)
    m[1, 2] = (top + bottom) / (top - bottom)
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2 * far * near / (far - near)
    m[3, 2] = -1.0
    return m  # row-major math matrix (float64)


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera world matrix of a camera at ``eye`` facing ``target`` (Matrix4.lookAt)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    z = eye - target
    if np.dot(z, z) == 0:
        z = np.array([0.0, 0.0, 1.0])
    z = z / np.linalg.norm(z)
    x = np.cross(up, z)
    if np.dot(x, x) == 0:
        z2 = z + np.array([1e-4, 0, 0]) if abs(up[2]) == 1 else z + np.array([0, 0, 1e-4])
        z = z2 / np.linalg.norm(z2)
        x = np.cross(up, z)
    x = x / np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = x, y, z, eye
    return m


def colmajor(m: np.ndarray) -> np.ndarray:
    return np.asarray(m, np.float64).T.reshape(-1)


def object_rows(camera_world: np.ndarray, object_worlds, visible=None) -> np.ndarray:
    """Object table rows (ObjectFrameState.ts:179-201), 40 floats per object."""
    view = np.linalg.inv(camera_world)
    cam_pos = camera_world[:3, 3]
    rows = np.zeros((len(object_worlds), 40), np.float64)
    for i, world in enumerate(object_worlds):
        world = np.asarray(world, np.float64)
        mv = view @ world
        local = np.linalg.inv(world) @ np.append(cam_pos, 1.0)
        rows[i, 0:16] = colmajor(world)
        rows[i, 16:32] = colmajor(mv)
        rows[i, 32:35] = local[:3]
        rows[i, 35] = 1.0
        rows[i, 36] = 1.0 if (visible is None or visible[i]) else 0.0
    return rows.astype(np.float32)


def make_frame(camera_world, width: int, height: int, fov_deg: float = 60.0, near: float = 0.1,
               far: float = 1000.0, object_worlds=None, **options) -> dict:
    """A frame description consumed by both the CUDA pipeline and the oracle."""
    if object_worlds is None:
        object_worlds = [np.eye(4)]
    proj = perspective(fov_deg, width / height, near, far)
    frame = {
        "projection": colmajor(proj).astype(np.float32),
        "view": colmajor(np.linalg.inv(camera_world)).astype(np.float32),
        "width": int(width), "height": int(height),
        "near": float(np.float32(near)), "far": float(np.float32(far)),
        "objects": object_rows(camera_world, object_worlds),
    }
    frame.update(options)
    return frame


# ---------------------------------------------------------------------------
# Seeded synthetic scenes (benchmark configurations).

def _unit_quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 3] < 0] *= -1
    return q.astype(np.float32)


def _sh(rng, n, degree, base=None):
    C = sh_coefficient_count(degree)
    sh = np.zeros((n, C, 3), np.float32)
    if base is None:
        base = rng.uniform(0, 1, (n, 3))
    sh[:, 0, :] = (base - 0.5) / SH_C0
    if C > 1:
        sh[:, 1:, :] = rng.normal(0, 0.1, (n, C - 1, 3))
    return sh


def uniform_cloud(n: int, seed: int = 1001, degree: int = 3, extent: float = 5.0,
                  log_scale=(-4.0, 0.5), opacity_logit=(0.0, 1.5), object_id: int = 0) -> dict:
    """Uniform-cube cloud: means U[-extent, extent]^3, ln-scales N(mu, s),
    opacity sigmoid(N(mu, s)), uniform unit quaternions, SH DC ~ U(0,1) and
    higher bands N(0, 0.1) (benchmark configuration 1 at n = 100k)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    means = rng.uniform(-extent, extent, (n, 3)).astype(np.float32)
    ls = rng.normal(log_scale[0], log_scale[1], (n, 3)).astype(np.float32)
    op = (1.0 / (1.0 + np.exp(-rng.normal(opacity_logit[0], opacity_logit[1], n)))).astype(np.float32)
    quats = _unit_quats(rng, n)
    sh = _sh(rng, n, degree)
    return pack_scene(means, np.full(n, object_id), ls, op, quats, sh)


def clustered_cloud(n: int, seed: int = 1002, degree: int = 3, clusters: int = 64,
                    centre_extent: float = 20.0, std=(0.2, 3.0), log_scale=(-3.5, 0.7),
                    opacity_logit=(0.5, 1.5), offset=(0.0, 0.0, 0.0),
                    degenerate_fraction: float = 0.0) -> dict:
    """Mixture of anisotropic Gaussian clusters (benchmark configurations 2 and 5)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-centre_extent, centre_extent, (clusters, 3))
    stds = rng.uniform(std[0], std[1], (clusters, 3))
    which = rng.integers(0, clusters, n)
    means = (centres[which] + rng.standard_normal((n, 3)) * stds[which] + np.asarray(offset)).astype(np.float32)
    ls = rng.normal(log_scale[0], log_scale[1], (n, 3)).astype(np.float32)
    if degenerate_fraction > 0:
        deg = rng.random(n) < degenerate_fraction
        axis = rng.integers(0, 3, n)
        ls[deg, axis[deg]] = -12.0
    op = (1.0 / (1.0 + np.exp(-rng.normal(opacity_logit[0], opacity_logit[1], n)))).astype(np.float32)
    quats = _unit_quats(rng, n)
    sh = _sh(rng, n, degree)
    return pack_scene(means, np.zeros(n), ls, op, quats, sh)


def orbit_cameras(count: int, radius: float = 30.0, seed: int = 1002, target=(0.0, 0.0, 0.0),
                  elevation_deg=(-30.0, 30.0)) -> list:
    """Seeded cameras on a sphere of ``radius`` around ``target`` looking at it."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    cams = []
    target = np.asarray(target, np.float64)
    for i in range(count):
        az = 2 * math.pi * (i + rng.uniform(0, 1)) / count
        el = math.radians(rng.uniform(*elevation_deg))
        eye = target + radius * np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
        cams.append(look_at(eye, target))
    return cams


def config1_scene(n: int = 100_000) -> dict:
    return uniform_cloud(n, seed=1001)


def config1_frame(**options) -> dict:
    return make_frame(look_at((0, 0, 15), (0, 0, 0)), 1280, 720, 60.0, 0.1, 1000.0, **options)


def config2_scene(n: int = 3_000_000) -> dict:
    return clustered_cloud(n, seed=1002)


def config2_frames(count: int = 16, width: int = 1920, height: int = 1080, **options) -> list:
    return [make_frame(c, width, height, 60.0, 0.1, 1000.0, **options)
            for c in orbit_cameras(count, 30.0, seed=1002)]


CONFIG3_SIZES = (50_000, 100_000, 250_000, 500_000, 750_000, 1_000_000, 1_500_000, 2_000_000)
CONFIG3_RESOLUTIONS = ((640, 480), (1280, 720), (1920, 1080), (3840, 2160))


def _rotation(rng) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def config3_scene(sizes=CONFIG3_SIZES, seed: int = 1003) -> tuple[dict, list]:
    """Benchmark configuration 3: one store holding the clouds as objects
    0..k-1 (configuration 1 distributions), and each object's world matrix: a
    seeded rigid transform with uniform scale U(0.5, 2), the clouds spread on
    a ring of radius 20."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = [uniform_cloud(n, seed=seed * 10 + i, object_id=i) for i, n in enumerate(sizes)]
    worlds = []
    for i in range(len(sizes)):
        m = np.eye(4)
        m[:3, :3] = _rotation(rng) * rng.uniform(0.5, 2.0)
        ang = 2 * math.pi * i / len(sizes)
        m[:3, 3] = (20.0 * math.cos(ang), rng.uniform(-3.0, 3.0), 20.0 * math.sin(ang))
        worlds.append(m)
    count = sum(p["count"] for p in parts)
    C = sh_coefficient_count(parts[0]["sh_degree"])
    sh = np.zeros(count * C + count, np.uint32)
    sh[: count * C] = np.concatenate([p["sh"][: p["count"] * C] for p in parts])
    sh[count * C:] = np.arange(count, dtype=np.uint32)
    scene = {"count": count, "active_count": count, "sh_degree": parts[0]["sh_degree"],
             "means": np.concatenate([p["means"] for p in parts]),
             "shape": np.concatenate([p["shape"] for p in parts]),
             "rotations": np.concatenate([p["rotations"] for p in parts]), "sh": sh}
    return scene, worlds


def config3_frames(worlds, count: int = 32, seed: int = 1003) -> list:
    """32 orbit cameras (radius 45 around the ring) with resolutions drawn
    from 640x480, 1280x720, 1920x1080 and 3840x2160."""
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    frames = []
    for cam_world in orbit_cameras(count, 45.0, seed=seed):
        w, h = CONFIG3_RESOLUTIONS[int(rng.integers(0, len(CONFIG3_RESOLUTIONS)))]
        frames.append(make_frame(cam_world, w, h, 60.0, 0.1, 1000.0, object_worlds=worlds))
    return frames
