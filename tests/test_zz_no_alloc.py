"""The allocation-free compaction entry point against the pipeline's own compaction.

gs3d_compact_visible_static keeps its scratch in a static device array so that
callers who cannot allocate device memory where they enqueue work (hosts with
their own memory arena, real-time loops that must not stall on the allocator)
can still run the visibility compaction. Its outputs must equal what gs3d_pipeline_render's
compaction stage produced for the same frame, on two calls in a row (the
second call finds the previous call's contents in the shared array).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import pkg, scenes
from gpu_harness import GpuRun

pytestmark = pytest.mark.gpu


def test_static_compaction_matches_pipeline_twice():
    import torch
    P = pkg()
    lib = P.load()
    sc = scenes()
    scene = sc.uniform_cloud(9000, seed=31, log_scale=(-2.4, 0.6))
    frame = sc.make_frame(sc.look_at((0.5, 1.0, 11.0), (0, 0, 0)), 200, 120, 55.0, 0.1, 100.0)
    run = GpuRun(scene, frame, "fp32")
    ref = run.render(frame)
    run.close()
    n = int(scene["active_count"])
    mean = ref["proj_mean"]
    visible = mean[:, 3] > 0
    keys_host = np.where(visible, mean[:, 2].view(np.uint32), np.uint32(0xFFFFFFFF)).astype(np.uint32)
    keys = torch.from_numpy(keys_host.view(np.int32)).cuda()
    for call in range(2):
        offs = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        kout = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        iout = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        result = torch.full((2,), -1, dtype=torch.int32, device="cuda")
        st = lib.gs3d_compact_visible_static(keys.data_ptr(), n, offs.data_ptr(), kout.data_ptr(), iout.data_ptr(),
                                             result.data_ptr(), None)
        assert st == 0, call
        torch.cuda.synchronize()
        count, err = (int(v) for v in result.cpu().numpy().view(np.uint32))
        assert err == 0
        assert count == int(ref["visible_state"][0]) == int(visible.sum())
        assert np.array_equal(offs.cpu().numpy().view(np.uint32), ref["visible_offsets"])
        ids = iout.cpu().numpy().view(np.uint32)[:count]
        ks = kout.cpu().numpy().view(np.uint32)[:count]
        assert np.array_equal(ids, np.nonzero(visible)[0].astype(np.uint32))
        order = np.argsort(ks, kind="stable")
        assert np.array_equal(np.stack([ks[order], ids[order]], 1), ref["depth_sorted"])


def test_static_compaction_rejects_oversize_and_null():
    lib = pkg().load()
    too_many = pkg().abi.STATIC_COMPACT_MAX_ITEMS + 1
    assert lib.gs3d_compact_visible_static(None, too_many, None, None, None, None, None) == 2
    assert lib.gs3d_compact_visible_static(None, 16, None, None, None, None, None) == 1


@pytest.mark.parametrize("pattern", ["random", "all", "none", "every7"])
def test_static_compaction_sizes(pattern):
    # The chunked compaction at sizes around its row (32), unit (256) and
    # chunk boundaries (a persistent grid of 4 blocks per SM: 608 chunks on a
    # GB300), from empty to multi-million inputs, against numpy.
    import torch
    lib = pkg().load()
    rng = np.random.Generator(np.random.PCG64(77))
    sizes = [0, 1, 2, 31, 32, 33, 255, 256, 257, 2047, 2048, 2049, 65535, 65537, 155647, 155648, 155649,
             1_000_003, 4_999_999]
    result = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    for n in sizes:
        if pattern == "random":
            vis = rng.random(n) < 0.5
        elif pattern == "all":
            vis = np.ones(n, bool)
        elif pattern == "none":
            vis = np.zeros(n, bool)
        else:
            vis = (np.arange(n) % 7) == 3
        keys_host = np.where(vis, rng.integers(0, 0xFFFFFFFE, n, dtype=np.uint32), np.uint32(0xFFFFFFFF))
        keys = torch.from_numpy(keys_host.astype(np.uint32).view(np.int32)).cuda() if n else None
        m = max(n, 1)
        offs = torch.full((m,), -1, dtype=torch.int32, device="cuda")
        kout = torch.full((m,), -1, dtype=torch.int32, device="cuda")
        iout = torch.full((m,), -1, dtype=torch.int32, device="cuda")
        st = lib.gs3d_compact_visible_static(keys.data_ptr() if n else None, n, offs.data_ptr(), kout.data_ptr(),
                                             iout.data_ptr(), result.data_ptr(), None)
        assert st == 0, n
        torch.cuda.synchronize()
        count, err = (int(v) for v in result.cpu().numpy().view(np.uint32))
        assert err == 0 and count == int(vis.sum()), n
        if n == 0:
            continue
        expect_off = (np.cumsum(vis) - vis).astype(np.uint32)
        assert np.array_equal(offs.cpu().numpy().view(np.uint32)[:n], expect_off), n
        idx = np.nonzero(vis)[0].astype(np.uint32)
        assert np.array_equal(iout.cpu().numpy().view(np.uint32)[:count], idx), n
        assert np.array_equal(kout.cpu().numpy().view(np.uint32)[:count], keys_host[idx]), n
