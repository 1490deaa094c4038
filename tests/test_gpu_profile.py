"""Profiling diagnostics (ProfileDiagnosticsStage.ts:22-116, utils/profileStats.ts:9-114,
kernels/profileDiagnostics.ts:8-64): the device-computed tile-load statistics,
cap estimates and zero-pixel subpixel count equal the reference's formulas
applied to the oracle's tile offsets and projected buffers."""
import ctypes as C
import importlib
import math

import numpy as np
import pytest

import oracle
from conftest import PKG_NAME
from gpu_harness import GpuRun

sc = importlib.import_module(PKG_NAME + ".scenes")
pytestmark = pytest.mark.gpu


def summarize(offsets):
    """summarizeTileLoads (utils/profileStats.ts:9-65)."""
    loads = np.maximum(np.diff(offsets.astype(np.int64)), 0)
    n = loads.size
    s = np.sort(loads)
    median = float(s[n // 2]) if n % 2 else (float(s[n // 2 - 1]) + float(s[n // 2])) * 0.5
    pct = lambda f: int(s[max(0, math.ceil(n * f) - 1)])
    batches = (loads + 255) // 256
    return {"max": int(loads.max()), "mean": float(loads.sum()) / n, "median": median, "p95": pct(0.95),
            "p99": pct(0.99), "tilesOver256": int((loads > 256).sum()), "tilesOver512": int((loads > 512).sum()),
            "tilesOver1024": int((loads > 1024).sum()), "tilesOver2048": int((loads > 2048).sum()),
            "totalBatches": int(batches.sum()), "maxBatches": int(batches.max())}


def estimate_cap(offsets, cap):
    """estimateTileCap (utils/profileStats.ts:67-100)."""
    loads = np.maximum(np.diff(offsets.astype(np.int64)), 0)
    r = np.minimum(loads, cap)
    d = loads - r
    emitted = int(r.sum() + d.sum())
    b = (r + 255) // 256
    return {"cap": cap, "rasterizedIntersections": int(r.sum()), "droppedIntersections": int(d.sum()),
            "droppedFraction": 0.0 if emitted == 0 else float(d.sum()) / emitted, "affectedTiles": int((d > 0).sum()),
            "totalBatches": int(b.sum()), "maxBatches": int(b.max())}


def zero_pixel(o, frame):
    L = oracle.lib()
    fp = C.POINTER(C.c_float)
    m = np.ascontiguousarray(o["proj_mean"], np.float32)
    c = np.ascontiguousarray(o["proj_conic"], np.float32)
    return sum(int(L.gso_zero_pixel_flag(m[i].ctypes.data_as(fp), c[i].ctypes.data_as(fp), frame["width"],
                                         frame["height"])) for i in range(m.shape[0]))


def cube(n, seed, log_scale):
    return sc.uniform_cloud(n, seed=seed, log_scale=log_scale)


CASES = {
    # Many subpixel splats (log-scale -5.5) among ordinary ones.
    "subpixel": (lambda: cube(20000, 81, (-5.0, 1.0)),
                 lambda: sc.make_frame(sc.look_at((0, 1, 12), (0, 0, 0)), 320, 200, 55.0, 0.1, 100.0)),
    # Heavy tiles (> 2048 records) and the configured raster cap.
    "heavy_capped": (lambda: cube(60000, 82, (-2.0, 0.5)),
                     lambda: sc.make_frame(sc.look_at((0, 0, 9), (0, 0, 0)), 128, 96, 60.0, 0.1, 100.0,
                                           max_splats_per_tile=1500)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_profile_stats_follow_the_reference_formulas(name):
    scene, frame = CASES[name][0](), CASES[name][1]()
    o = oracle.render(scene, frame, 0, output_depth=False)
    run = GpuRun(scene, frame, "fp32", capacity=max(int(o["state"][1]), 1))
    g = run.render(frame)
    prof = run.pipe.read_profile()
    run.close()
    assert np.array_equal(g["tile_offsets"], o["tile_offsets"])  # same input as the formulas below
    want = summarize(o["tile_offsets"])
    for k, v in want.items():
        assert prof["tileLoads"][k] == pytest.approx(v, rel=0, abs=1e-9), k
    for got, cap in zip(prof["tileCapEstimates"], (2048, 4096, 8192)):
        assert got == pytest.approx(estimate_cap(o["tile_offsets"], cap))
    cap = int(frame.get("max_splats_per_tile", 0))
    if cap:
        assert prof["appliedTileCap"] == pytest.approx(estimate_cap(o["tile_offsets"], cap))
        assert want["tilesOver2048"] > 0
    else:
        assert prof["appliedTileCap"] is None
    assert prof["zeroPixelSubpixelSplats"] == zero_pixel(o, frame)
    if name == "subpixel":
        assert prof["zeroPixelSubpixelSplats"] > 0
