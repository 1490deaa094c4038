"""The object-transform table and the multi-cloud, multi-view workload against the oracle.

The reference writes, per cloud and frame, the world matrix, the model-view
matrix, the camera position in object space and a visible flag
(src/renderer/pipeline/ObjectFrameState.ts:97-119); the projection reads the
row of each splat's object (ProjectionStage.ts:429-450) and takes the SH view
direction from the camera position in object space (:469). These tests use
the multi-cloud workload (eight clouds with the single-cloud distributions,
each with a seeded rigid transform and a uniform scale in U(0.5, 2)) at 1/50
of its splat counts, with one hidden object, splats whose object id has no
row, views from 640x480 to 3840x2160, single views and one batch of two view
groups. The EXACT form is compared bit for bit (every buffer and the image);
the half2 form keeps every integer buffer bit-exact and is held to
>= 50 dB against the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import scenes
from gpu_harness import GpuRun, assert_bit_exact, psnr, render_batch

gpu = pytest.mark.gpu

sc = scenes()
SIZES = tuple(n // 50 for n in sc.CONFIG3_SIZES)  # 1000 ... 40000 splats per cloud
HIDDEN = 3          # object whose visible flag is 0
ORPHAN_ID = 8.0     # object id past the 8-row table
MIN_PSNR_DB = 50.0
HALF2_MAX_ABS = 2e-2


def scene_with_edge_objects(seed=1003):
    scene, worlds = sc.config3_scene(SIZES, seed=seed)
    means = scene["means"]
    rng = np.random.Generator(np.random.PCG64(seed + 5))
    orphans = rng.choice(scene["count"], 300, replace=False)
    means[orphans, 3] = ORPHAN_ID
    return scene, worlds


def frame_for(worlds, eye, width, height, hidden=HIDDEN):
    frame = sc.make_frame(sc.look_at(eye, (0.0, 0.0, 0.0)), width, height, 60.0, 0.1, 1000.0, object_worlds=worlds)
    if hidden is not None:
        frame["objects"][hidden, 36] = 0.0
    return frame


SCENE, WORLDS = scene_with_edge_objects()
EYES = [(0.0, 8.0, 45.0), (31.8, -6.0, 31.8), (-44.0, 12.0, 9.0), (5.0, 40.0, -20.0)]


def test_object_rows_reach_the_projection():
    # (CPU, oracle only) The table is not a no-op: the hidden object and the
    # orphan splats draw nothing, every other object draws, and moving one
    # object moves its splats only.
    frame = frame_for(WORLDS, EYES[0], 640, 480)
    o = oracle.render(SCENE, frame, 0)
    obj = SCENE["means"][:, 3]
    drawn = o["tile_counts"] > 0
    assert not drawn[obj == HIDDEN].any()
    assert not drawn[obj == ORPHAN_ID].any()
    for k in range(len(SIZES)):
        if k != HIDDEN:
            assert drawn[obj == k].any(), k
    moved = [w.copy() for w in WORLDS]
    moved[5][:3, 3] += np.array([0.7, 0.0, 0.0])
    o2 = oracle.render(SCENE, frame_for(moved, EYES[0], 640, 480), 0)
    changed = np.any(o["proj_mean"] != o2["proj_mean"], axis=1)
    assert changed[obj == 5].any() and not changed[obj != 5].any()


@gpu
@pytest.mark.parametrize("view", [(0, 640, 480), (1, 1280, 720), (2, 1920, 1080), (3, 3840, 2160)])
def test_single_view_bit_exact(view):
    i, w, h = view
    frame = frame_for(WORLDS, EYES[i], w, h)
    o = oracle.render(SCENE, frame, 0)
    assert int(o["state"][1]) > 0
    run = GpuRun(SCENE, frame, "exact", capacity=int(o["state"][1]) + 256)
    g = run.render(frame)
    run.close()
    assert_bit_exact(g, o)


@gpu
def test_every_object_visible_and_scaled_rows():
    # No hidden object: all eight transformed clouds (scales 0.5..2) draw.
    frame = frame_for(WORLDS, EYES[1], 1280, 720, hidden=None)
    o = oracle.render(SCENE, frame, 0)
    run = GpuRun(SCENE, frame, "exact", capacity=int(o["state"][1]) + 256)
    g = run.render(frame)
    run.close()
    assert_bit_exact(g, o)


def second_scene():
    scene, worlds = sc.config3_scene(tuple(n // 2 for n in SIZES[:4]), seed=2003)
    return scene, worlds


def batch_pairs():
    # Two view groups: three views of the first store (one at 3840x2160),
    # then two of a second store; mixed resolutions.
    scene2, worlds2 = second_scene()
    return [(SCENE, frame_for(WORLDS, EYES[0], 640, 480)),
            (SCENE, frame_for(WORLDS, EYES[2], 3840, 2160)),
            (SCENE, frame_for(WORLDS, EYES[3], 1280, 720)),
            (scene2, frame_for(worlds2, EYES[1], 1920, 1080, hidden=1)),
            (scene2, frame_for(worlds2, EYES[0], 800, 600, hidden=None))]


@gpu
def test_batch_of_two_view_groups_bit_exact():
    pairs = batch_pairs()
    views, stats = render_batch(pairs, "exact", share_scenes=True)
    total = 0
    for (scene, frame), g in zip(pairs, views):
        o = oracle.render(scene, frame, 0)
        total += int(o["state"][0])
        vis = o["tile_counts"] > 0
        assert np.array_equal(g["tile_counts"], o["tile_counts"])
        assert np.array_equal(g["proj_mean"].view(np.uint32), o["proj_mean"].view(np.uint32))
        assert np.array_equal(g["proj_conic"][vis].view(np.uint32), o["proj_conic"][vis].view(np.uint32))
        assert np.array_equal(g["proj_color"][vis].view(np.uint32), o["proj_color"][vis].view(np.uint32))
        assert np.array_equal(g["visible_offsets"], o["visible_offsets"])
        assert np.array_equal(g["depth_sorted"], o["depth_sorted"])
        assert np.array_equal(g["ordered_counts"], o["ordered_counts"])
        assert np.array_equal(g["sorted_records"], o["sorted_records"])
        assert np.array_equal(g["tile_offsets"], o["tile_offsets"])
        assert np.array_equal(g["rgba"].view(np.uint32), o["rgba"].view(np.uint32))
        assert np.array_equal(g["depth"].view(np.uint32), o["depth"].view(np.uint32))
    assert stats["intersectionCount"] == total


@gpu
def test_batch_half2_integer_exact_and_psnr():
    pairs = batch_pairs()
    views, _ = render_batch(pairs, "half2", share_scenes=True)
    for (scene, frame), g in zip(pairs, views):
        o = oracle.render(scene, frame, 0)
        o64 = oracle.render(scene, frame, 1)
        assert np.array_equal(g["tile_counts"], o["tile_counts"])
        assert np.array_equal(g["proj_mean"].view(np.uint32), o["proj_mean"].view(np.uint32))
        assert np.array_equal(g["depth_sorted"], o["depth_sorted"])
        assert np.array_equal(g["sorted_records"], o["sorted_records"])
        assert np.array_equal(g["tile_offsets"], o["tile_offsets"])
        assert np.abs(g["rgba"] - o["rgba"]).max() <= HALF2_MAX_ABS
        assert psnr(g["rgba"][..., :3], o64["rgba"][..., :3]) >= MIN_PSNR_DB
