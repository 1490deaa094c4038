"""Writes the golden fixtures under tests/golden/.

known_answers.json
    The reference test suite's own known-answer vectors, transcribed with the
    file:line they come from. When the reference checkout is available
    (``--reference DIR``), every transcribed literal is checked to appear in
    the cited test file, so the fixture cannot drift from its source.

small_scene.npz
    A seeded 3000-splat scene and frames, plus the FP32 oracle's integer
    outputs (tile counts, visible offsets, depth-sorted records, intersection
    offsets, sorted intersection records, tile offsets) and images. GPU tests
    compare the CUDA path with these committed vectors as well as with a
    fresh oracle run.

Usage: python tests/golden/make_golden.py [--reference /path/to/3dgs_tile_webgpu]
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

KNOWN_ANSWERS = {
    "perspective_default": {
        "source": "test/ProjectionBoundary.test.ts:30-54",
        "view": [0.0, 0.0, -2.0],
        "clipped_view": [0.0, 0.0, 2.0],
        "viewport": [32.0, 32.0, 1.0, 10.0],
        "filter": 0.3,
        "center_depth": [16.0, 16.0, 2.0],
        "cov_xx": 64.3,
        "unfiltered_det": 4096.0,
    },
    "projection_result": {
        "source": "test/ProjectionBoundary.test.ts:56-72",
        "center": [-3.0, 7.0],
        "depth": 42.0,
        "cov": [4.0, 1.0, 9.0],
    },
    "periodic_delta": {
        "source": "test/ProjectionBoundary.test.ts:74-104",
        "conic": [0.1, 0.08, 0.12],
        "viewport": [7.0, 9.0],
        "center": [-15.25, 26.5],
        "pixels": [[0.5, 0.5], [6.5, 8.5], [3.5, 4.5]],
    },
    "tile_hit_fixtures": [
        {"source": "test/ProjectionBoundary.test.ts:107", "center": [-0.25, 8.5], "cov": [4, 0, 4],
         "width": 33, "height": 17, "axis": 1},
        {"source": "test/ProjectionBoundary.test.ts:108", "center": [16.5, 18.25], "cov": [4, 0, 4],
         "width": 33, "height": 17, "axis": 2},
        {"source": "test/ProjectionBoundary.test.ts:109", "center": [-35.5, 8.5], "cov": [100, 24, 9],
         "width": 7, "height": 17, "axis": 1},
        {"source": "test/ProjectionBoundary.test.ts:110", "center": [8.5, -41.25], "cov": [9, 24, 100],
         "width": 17, "height": 7, "axis": 2},
    ],
    "subpixel": {
        "source": "test/ProjectionBoundary.test.ts:165-175",
        "center": [33.5, 0.5], "conic": [100.0, 0.0, 100.0], "thr": 1.0, "extent": [0.1, 0.1],
        "viewport": [33, 17], "expected": [1, 0],
    },
    "finalize_depth": {
        "source": "test/ScalarOutput.test.ts:61-97",
        "invalid": [[0.0, 1.0], [0.6, 0.8], [float("inf"), 0.1], [float("nan"), 0.1], [0.0, 0.1]],
        "finite": [[8.8, 0.2], [880.0, 0.2]],
        "finite_expected": [11.0, 1100.0],
    },
    "sh_round_trip": [[0, 0, 0], [1, -0.5, 0.25], [-3.75, 2.125, 0.03125], [1e-4, -2e-4, 3e-4]],
    "sh_round_trip_source": "test/GaussianSh.test.ts:19-41",
    "compact_geometry": [
        {"source": "rust/gaussian-backend/tests/backend.rs:1089-1093",
         "position": [123456.75, -0.000123, 32.5], "scale": [1e-8, 1.234, 1e5],
         # Quat::from_rotation_y(2.4) = (0, sin 1.2, 0, cos 1.2)
         "quat": [0.0, 0.9320390859672263, 0.0, 0.3623577544766736], "opacity": 0.73},
        {"source": "rust/gaussian-backend/tests/backend.rs:1095",
         "position": [-2.0, 0.0, 0.0], "scale": [0.2, 0.2, 0.2], "quat": [0.0, 0.0, 0.0, 1.0],
         "opacity": 0.73},
    ],
    "chunk_composite": [
        {"color": [0.8, 0.1, 0.2], "alpha": 0.25},
        {"color": [0.2, 0.7, 0.3], "alpha": 0.4},
        {"color": [0.1, 0.2, 0.9], "alpha": 0.15},
        {"color": [0.9, 0.8, 0.1], "alpha": 0.35},
    ],
    "chunk_composite_source": "test/rasterizationWGSL.test.ts:63-86",
}

# Literal snippets that must appear in the cited reference files.
PROVENANCE = [
    ("test/ProjectionBoundary.test.ts", ["vec3<f32>(0.0,0.0,-2.0)", "vec4<f32>(32.0,32.0,1.0,10.0), 0.3",
                                         "toBeCloseTo(64.3, 4)", "toBe(4096)", "vec3<f32>(0.0,0.0,2.0)",
                                         "vec2<f32>(-3.0,7.0), 42.0, vec3<f32>(4.0,1.0,9.0), 0.0",
                                         "[0.1, 0.08, 0.12]", "[7, 9]", "[-15.25, 26.5]",
                                         "center: [-0.25, 8.5], cov: [4, 0, 4], width: 33, height: 17, axis: 1",
                                         "center: [16.5, 18.25], cov: [4, 0, 4], width: 33, height: 17, axis: 2",
                                         "center: [-35.5, 8.5], cov: [100, 24, 9], width: 7, height: 17, axis: 1",
                                         "center: [8.5, -41.25], cov: [9, 24, 100], width: 17, height: 7, axis: 2",
                                         "vec2<f32>(33.5,0.5),vec3<f32>(100.0,0.0,100.0),1.0,vec2<f32>(0.1),vec2<u32>(33u,17u),1u"]),
    ("test/ScalarOutput.test.ts", ["[0.6, 0.8]", "[8.8, 0.2]", "[880, 0.2]", "toBeCloseTo(11, 5)",
                                   "toBeCloseTo(1100, 3)"]),
    ("test/GaussianSh.test.ts", ["[1, -0.5, 0.25]", "[-3.75, 2.125, 0.03125]", "[1e-4, -2e-4, 3e-4]"]),
    ("rust/gaussian-backend/tests/backend.rs", ["Vec3A::new(123456.75, -0.000123, 32.5)",
                                                "Vec3A::new(1e-8, 1.234, 1e5)", "Quat::from_rotation_y(2.4)",
                                                "0.73", "< 0.01", "< 0.001", "> 0.99999"]),
    ("test/rasterizationWGSL.test.ts", ["[0.8, 0.1, 0.2], alpha: 0.25", "[0.2, 0.7, 0.3], alpha: 0.4",
                                        "[0.1, 0.2, 0.9], alpha: 0.15", "[0.9, 0.8, 0.1], alpha: 0.35"]),
]


def check_provenance(reference: str) -> None:
    for rel, snippets in PROVENANCE:
        with open(os.path.join(reference, rel)) as f:
            text = f.read()
        for snip in snippets:
            if snip not in text:
                raise SystemExit(f"{rel}: '{snip}' not found")


def small_scene_cases():
    sc = importlib.import_module("3dgs_tile_webgpu_gb300.scenes")
    scene = sc.uniform_cloud(3000, seed=4242, log_scale=(-2.5, 0.6))
    rng = np.random.Generator(np.random.PCG64(99))
    # Exercise the active-slot tail and empty slots: a shuffled subset.
    active = rng.permutation(scene["count"])[:2600].astype(np.uint32)
    scene["sh"][scene["count"] * 16: scene["count"] * 16 + active.size] = active
    scene["active_count"] = int(active.size)
    scene["means"][rng.choice(scene["count"], 50, replace=False), 3] = -1.0
    frames = {
        "front": sc.make_frame(sc.look_at((0, 0, 12), (0, 0, 0)), 160, 96, 60.0, 0.1, 100.0,
                               raster_chunk_size=8192),
        "oblique": sc.make_frame(sc.look_at((6, 4, 9), (0, 0.5, 0)), 131, 77, 50.0, 0.5, 40.0,
                                 raster_chunk_size=256, background=(0.2, 0.3, 0.4, 0.5)),
    }
    return scene, frames


def write_small_scene() -> None:
    import oracle
    scene, frames = small_scene_cases()
    arrays = {f"scene_{k}": np.asarray(v) for k, v in scene.items()}
    for name, fr in frames.items():
        res = oracle.render(scene, fr, 0)
        for key in ("tile_counts", "visible_offsets", "depth_sorted", "intersection_offsets",
                    "sorted_records", "tile_offsets", "state", "visible_state"):
            arrays[f"{name}_{key}"] = np.asarray(res[key])
        arrays[f"{name}_rgba"] = res["rgba"].astype(np.float16)
    np.savez_compressed(os.path.join(HERE, "small_scene.npz"), **arrays)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    args = ap.parse_args()
    if args.reference:
        check_provenance(args.reference)
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(KNOWN_ANSWERS, f, indent=1)
    write_small_scene()


if __name__ == "__main__":
    main()
