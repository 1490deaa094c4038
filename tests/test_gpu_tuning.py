"""Launch-shape tuning (gs3d_tuning, no counterpart in the reference): views
per launch, tile-sort digit width and raster work order change how the batch
is launched, never what it produces; the autotuner picks among them and the
tile size (tests/test_gpu_tile_size.py covers the tile size itself)."""
import importlib

import numpy as np
import pytest

from conftest import PKG_NAME

P = importlib.import_module(PKG_NAME)
dev = importlib.import_module(PKG_NAME + ".device")
sc = importlib.import_module(PKG_NAME + ".scenes")

pytestmark = pytest.mark.gpu


def cam(eye=(0.0, 0.0, 11.0), w=160, h=96):
    return sc.make_frame(sc.look_at(eye, (0.0, 0.0, 0.0)), w, h, 60.0, 0.1, 100.0)


def batch():
    clouds = [sc.uniform_cloud(5000, seed=71, log_scale=(-2.4, 0.6)),
              sc.uniform_cloud(3000, seed=72, log_scale=(-2.0, 0.5)),
              sc.uniform_cloud(4000, seed=73, degree=1, log_scale=(-2.4, 0.6))]
    frames = [cam(w=200, h=120), cam(eye=(3, 2, 9), w=97, h=64), cam(eye=(-4, 1, 10), w=160, h=96),
              cam(eye=(0, 6, 8), w=33, h=17), cam(w=128, h=128), cam(eye=(2, -3, 9), w=64, h=200)]
    pairs = [(clouds[i % 3], f) for i, f in enumerate(frames)]
    return pairs


class Batch:
    def __init__(self, pairs, precision="exact", capacity=1 << 22):
        import torch
        self.dss = [dev.DeviceScene(s) for s, _ in pairs]
        self.pipe = P.TiledGaussianPipeline(self.dss[0].data(), {"raster_precision": precision,
                                                                  "intersection_capacity": capacity})
        self.colors, self.views = [], []
        for ds, (scene, frame) in zip(self.dss, pairs):
            W, H = int(frame["width"]), int(frame["height"])
            color = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
            self.colors.append(color)
            self.views.append((ds.data(), P.make_camera(frame), W, H, color.data_ptr(), 0, "rgba32f"))

    def render(self, tuning=None):
        import torch
        if tuning is not None:
            self.pipe.set_tuning(tuning)
        for c in self.colors:
            c.fill_(-1.0)
        self.pipe.render_batch(self.views)
        stats = self.pipe.read_stats()
        torch.cuda.synchronize()
        return [c.cpu().numpy() for c in self.colors], stats

    def close(self):
        self.pipe.dispose()


def same_images(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def test_views_per_launch_gives_the_same_images_and_summed_counts():
    b = Batch(batch())
    ref, st = b.render({"views_per_launch": 0})
    for per in (4, 2, 1):
        imgs, s = b.render({"views_per_launch": per})
        assert same_images(imgs, ref), per
        assert s["visibleGaussianCount"] == st["visibleGaussianCount"]
        assert s["intersectionCount"] == st["intersectionCount"]
        assert not s["overflow"]
        assert s["requestedIntersections"] <= st["requestedIntersections"]  # largest launch sequence
    b.close()


@pytest.mark.parametrize("digits", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("order", [0, 1])
def test_tile_digit_width_and_work_order_change_nothing(digits, order):
    b = Batch(batch())
    ref, _ = b.render({"views_per_launch": 0, "tile_digit_bits": 8, "work_order": 1})
    imgs, _ = b.render({"tile_digit_bits": digits, "work_order": order})
    assert same_images(imgs, ref)
    b.close()


def test_narrow_tile_digits_on_many_tiles_stay_within_four_passes():
    # Over 2^16 tiles (19-bit tile ids): 4-bit digits would need 5 passes; the
    # sort caps the passes at the 4 its histograms hold and widens the digit.
    clouds = [sc.uniform_cloud(3000, seed=74, log_scale=(-2.0, 0.5))]
    frames = [cam(w=4096, h=4096), cam(eye=(2, 1, 10), w=4096, h=4096), cam(eye=(-2, 1, 9), w=4096, h=2048)]
    pairs = [(clouds[0], f) for f in frames]
    b = Batch(pairs)
    ref, st = b.render({"tile_digit_bits": 8})
    imgs, s = b.render({"tile_digit_bits": 4})
    assert same_images(imgs, ref)
    assert s["intersectionCount"] == st["intersectionCount"] and s["deviceError"] == 0
    b.close()


def test_chunked_batch_overflow_is_reported_for_the_batch():
    pairs = batch()
    b = Batch(pairs, capacity=1 << 22)
    _, st = b.render({"views_per_launch": 2})
    need = st["requestedIntersections"]
    b.pipe.resize_intersections(max(need // 2, 256))
    _, s = b.render()
    assert s["overflow"]
    r = b.pipe.get_resources()
    out = dev.to_numpy(r.output_state, (4,))
    assert out[3] == 1 and out[2] == s["requestedIntersections"]
    b.close()


def test_chunked_graph_replay_matches_direct_batches():
    import torch
    b = Batch(batch())
    b.pipe.set_tuning({"views_per_launch": 2})
    ref, st = b.render()
    stream = torch.cuda.Stream()
    b.pipe.capture_graph(b.views, stream.cuda_stream)
    for c in b.colors:
        c.fill_(-1.0)
    with torch.cuda.stream(stream):
        b.pipe.launch_graph([v[1] for v in b.views], stream=stream.cuda_stream)
    stream.synchronize()
    assert same_images([c.cpu().numpy() for c in b.colors], ref)
    s = b.pipe.read_stats()
    assert s["visibleGaussianCount"] == st["visibleGaussianCount"]
    assert s["intersectionCount"] == st["intersectionCount"]
    b.close()


def test_autotune_picks_a_valid_tuning_and_keeps_the_images():
    b = Batch(batch(), precision="half2")
    ref, _ = b.render()
    tuning, ms = b.pipe.autotune(b.views, trials=2)
    assert ms > 0.0
    assert 4 <= tuning["tile_digit_bits"] <= 8 and tuning["work_order"] in (0, 1)
    assert tuning["views_per_launch"] in (0, 3, 1)  # halving from 6 views: 3, then 1
    assert tuning["tile_size"] in (8, 16, 32) and tuning["raster_pixels_per_lane"] in (2, 4)
    imgs, _ = b.render()
    for x, y in zip(imgs, ref):
        if tuning["tile_size"] == 16 and tuning["raster_pixels_per_lane"] == 2:  # same images
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        else:  # other tiles or patches regroup each pixel's records: within the half2 tolerance
            assert np.abs(x - y).max() <= 2e-2
    b.close()


def test_invalid_tuning_is_rejected():
    b = Batch(batch()[:1])
    with pytest.raises(ValueError):
        b.pipe.set_tuning({"tile_digit_bits": 3})
    with pytest.raises(ValueError):
        b.pipe.set_tuning({"tile_digit_bits": 9})
    b.close()
