"""The continuous-batching server: every image equals the same request rendered
alone (views of a batch are independent), across lanes, batch sizes and
overflow retries."""
import importlib

import numpy as np
import pytest

from conftest import PKG_NAME, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "half2"])
def test_results_same_alone_and_in_the_mix(precision):
    import torch
    P = importlib.import_module(PKG_NAME)
    dev = importlib.import_module(PKG_NAME + ".device")
    srv_mod = importlib.import_module(PKG_NAME + ".serving")
    sc = scenes()
    clouds = {"a": dev.DeviceScene(sc.uniform_cloud(6000, seed=51, log_scale=(-2.4, 0.6))),
              "b": dev.DeviceScene(sc.clustered_cloud(20000, seed=52, clusters=8, centre_extent=4.0,
                                                      log_scale=(-3.0, 0.6)))}
    rng = np.random.Generator(np.random.PCG64(5))
    sizes = [(160, 96), (97, 64), (200, 120)]
    reqs = []
    for i in range(24):
        name = "a" if i % 3 else "b"
        w, h = sizes[i % 3]
        eye = rng.uniform(-1, 1, 3) * 3 + np.array([0.0, 0.0, 11.0])
        frame = sc.make_frame(sc.look_at(eye, (0, 0, 0)), w, h, 55.0, 0.1, 100.0)
        reqs.append(srv_mod.Request(i, name, frame))
    # Tiny initial capacity: the first batches overflow and are retried.
    server = srv_mod.RenderServer(clouds, lanes=2, budget_bytes=2e9, max_views=5, precision=precision,
                                  initial_capacity=1024)
    stats = server.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and stats["retries"] >= 1
    for r in reqs:
        alone = P.TiledGaussianPipeline(clouds[r.scene].data(), {"raster_precision": precision,
                                                                  "intersection_capacity": 1 << 20})
        W, H = r.frame["width"], r.frame["height"]
        alone.prepare_frame(W, H)
        img = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
        alone.render(P.make_camera(r.frame), img.data_ptr(), 0, color_format="rgba16f")
        torch.cuda.synchronize()
        assert torch.equal(img, r.color), r.rid
        alone.dispose()
    server.close()


def test_closed_loop_keeps_concurrency_and_results():
    # Closed loop with 12 requests outstanding over two lanes: every request
    # completes once, latencies are recorded after the warm-up, and images
    # equal the request rendered alone.
    import torch
    P = importlib.import_module(PKG_NAME)
    dev = importlib.import_module(PKG_NAME + ".device")
    srv_mod = importlib.import_module(PKG_NAME + ".serving")
    sc = scenes()
    clouds = {"a": dev.DeviceScene(sc.uniform_cloud(5000, seed=53, log_scale=(-2.4, 0.6))),
              "b": dev.DeviceScene(sc.uniform_cloud(8000, seed=54, log_scale=(-2.6, 0.6)))}
    rng = np.random.Generator(np.random.PCG64(6))
    made = []

    def make_request(i):
        name = "a" if i % 2 else "b"
        w, h = [(160, 96), (128, 128)][i % 2]
        eye = rng.uniform(-1, 1, 3) * 3 + np.array([0.0, 0.0, 11.0])
        r = srv_mod.Request(i, name, sc.make_frame(sc.look_at(eye, (0, 0, 0)), w, h, 55.0, 0.1, 100.0))
        made.append(r)
        return r

    server = srv_mod.RenderServer(clouds, lanes=2, budget_bytes=2e9, max_views=4, precision="half2",
                                  initial_capacity=1 << 16)
    stats = server.run_closed(make_request, concurrency=12, total=40, warmup=12)
    assert stats["requests"] == 40 and stats["p99_ms"] >= stats["p50_ms"] > 0
    assert len(made) == 52 and all(r.completed >= r.arrival > 0 for r in made)
    for r in made[::5]:
        alone = P.TiledGaussianPipeline(clouds[r.scene].data(), {"raster_precision": "half2",
                                                                  "intersection_capacity": 1 << 20})
        W, H = r.frame["width"], r.frame["height"]
        alone.prepare_frame(W, H)
        img = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
        alone.render(P.make_camera(r.frame), img.data_ptr(), 0, color_format="rgba16f")
        torch.cuda.synchronize()
        assert torch.equal(img, r.color), r.rid
        alone.dispose()
    server.close()
