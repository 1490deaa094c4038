"""Failure paths of the output-status machine, made to happen without a GPU fault.

* A look-back wait that runs out: the compaction's first chunk is withheld
  (a status word that nothing publishes), a short wait limit expires, the
  kernel finishes, the frame reports GS3D_ERROR_DEVICE_TIMEOUT and the same
  pipeline renders the next frame bit-exact.
* "allocation-failed" (types.ts:209-233, GaussianPass.ts:808-826): a device
  allocation is made to fail on the host; the call returns
  GS3D_ERROR_OUT_OF_MEMORY, the previous workspaces stay, and the pipeline
  keeps rendering bit-exact.
* The asynchronous stats read-back (GaussianPass.ts:1019-1079) returns what
  the synchronous read returns, one read-back in flight at a time.
"""
import time

import numpy as np
import pytest

import oracle
from conftest import pkg, scenes
from gpu_harness import GpuRun, assert_bit_exact

pytestmark = pytest.mark.gpu

sc = scenes()


def case(seed=71, n=6000):
    scene = sc.uniform_cloud(n, seed=seed, log_scale=(-2.4, 0.6))
    frame = sc.make_frame(sc.look_at((0.5, 1.0, 11.0), (0, 0, 0)), 200, 120, 55.0, 0.1, 100.0)
    return scene, frame


def render_raw(run, frame):
    """Enqueue one render without reading anything back."""
    import torch
    P = pkg()
    W, H = int(frame["width"]), int(frame["height"])
    run.pipe.prepare_frame(W, H)
    color = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    run.pipe.render(P.make_camera(frame), color.data_ptr(), 0, 1, False, "rgba32f")
    return color


def test_lookback_wait_expires_and_pipeline_recovers():
    P = pkg()
    scene, frame = case()
    o = oracle.render(scene, frame, 0)
    run = GpuRun(scene, frame, "exact", capacity=int(o["state"][1]) + 256)
    run.pipe.set_wait_limit(2000)  # a few hundred microseconds of polling
    run.pipe.debug_withhold_chunk()
    t0 = time.time()
    render_raw(run, frame)
    with pytest.raises(P.GaussianPassError) as err:
        run.pipe.read_stats()
    assert err.value.status == P.abi.GS3D_ERROR_DEVICE_TIMEOUT
    assert time.time() - t0 < 30.0  # the kernel returned on its own
    # The hook applies to one render only; the next frame is complete and exact.
    g = run.render(frame)
    assert g["stats"]["deviceError"] == 0
    assert_bit_exact(g, o)
    # The default limit again: still exact.
    run.pipe.set_wait_limit(0)
    assert_bit_exact(run.render(frame), o)
    run.close()


def test_allocation_failure_keeps_previous_workspaces():
    P = pkg()
    scene, frame = case(seed=72)
    o = oracle.render(scene, frame, 0)
    need = int(o["state"][1])
    run = GpuRun(scene, frame, "exact", capacity=need + 256)
    assert_bit_exact(run.render(frame), o)
    # Intersection workspaces: the second of the four new buffers fails.
    P.debug_fail_allocation(2)
    with pytest.raises(P.GaussianPassError) as err:
        run.pipe.resize_intersections(4 * need)
    assert err.value.status == P.abi.GS3D_ERROR_OUT_OF_MEMORY
    g = run.render(frame)
    assert g["stats"]["intersectionCapacity"] == need + 256
    assert_bit_exact(g, o)
    # Per-splat workspaces: a larger store whose growth fails part-way.
    dev = __import__(P.__name__ + ".device", fromlist=["DeviceScene"])
    big = dev.DeviceScene(sc.uniform_cloud(40000, seed=73, log_scale=(-2.4, 0.6)))
    P.debug_fail_allocation(5)
    with pytest.raises(P.GaussianPassError) as err:
        run.pipe.update_data(big.data())
    assert err.value.status == P.abi.GS3D_ERROR_OUT_OF_MEMORY
    assert_bit_exact(run.render(frame), o)
    # With the hook spent, growth succeeds and the frame is still exact.
    P.debug_fail_allocation(0)
    run.pipe.resize_intersections(4 * need)
    assert_bit_exact(run.render(frame), o)
    run.close()


def test_async_stats_match_synchronous_read():
    P = pkg()
    scene, frame = case(seed=74)
    run = GpuRun(scene, frame, "fp32", capacity=1 << 20)
    render_raw(run, frame)
    run.pipe.request_stats()
    with pytest.raises(P.GaussianPassError):
        run.pipe.request_stats()  # one read-back in flight
    got = run.pipe.poll_stats(wait=False)
    if got is None:
        got = run.pipe.poll_stats(wait=True)
    assert got == run.pipe.read_stats()
    assert got["visibleGaussianCount"] > 0 and got["intersectionCount"] > 0
    # A batch rendered as several launch sequences reports its totals.
    run.pipe.set_tuning({"views_per_launch": 1})
    import torch
    colors = [torch.zeros((120, 200, 4), dtype=torch.float32, device="cuda") for _ in range(3)]
    cams = [P.make_camera(sc.make_frame(sc.look_at((x, 1.0, 11.0), (0, 0, 0)), 200, 120, 55.0, 0.1, 100.0))
            for x in (-1.0, 0.0, 1.0)]
    run.pipe.render_batch([(run.ds.data(), c, 200, 120, col.data_ptr(), 0, "rgba32f") for c, col in zip(cams, colors)])
    run.pipe.request_stats()
    got = run.pipe.poll_stats(wait=True)
    assert got == run.pipe.read_stats()
    # A frame whose look-back wait ran out reports it through the poll too.
    run.pipe.set_tuning({"views_per_launch": 0})
    run.pipe.set_wait_limit(2000)
    run.pipe.debug_withhold_chunk()
    render_raw(run, frame)
    run.pipe.request_stats()
    with pytest.raises(P.GaussianPassError) as err:
        run.pipe.poll_stats(wait=True)
    assert err.value.status == P.abi.GS3D_ERROR_DEVICE_TIMEOUT
    with pytest.raises(P.GaussianPassError):
        run.pipe.poll_stats(wait=True)  # nothing requested any more
    run.close()
