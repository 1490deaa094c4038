"""Accuracy of the deterministic math library and invariants of the oracle pass."""
import importlib

import numpy as np
import pytest

import oracle

sc = importlib.import_module("3dgs_tile_webgpu_gb300.scenes")


def ulp_err(got: np.ndarray, exact: np.ndarray) -> float:
    exact32 = exact.astype(np.float32)
    spacing = np.spacing(np.abs(exact32)).astype(np.float64)
    return float(np.max(np.abs(got.astype(np.float64) - exact) / spacing))


@pytest.mark.parametrize("name,fn,lo,hi,max_ulp", [
    ("expf", np.exp, -20.0, 12.0, 2.0),
    ("expf", np.exp, -1e-3, 1e-3, 2.0),
    ("logf", np.log, 1e-6, 1e6, 2.0),
    ("logf", np.log, 0.5, 2.0, 2.0),
    ("sinf", np.sin, -1.6, 1.6, 2.0),
    ("cosf", np.cos, -1.6, 1.6, 2.0),
])
def test_unary_accuracy(name, fn, lo, hi, max_ulp):
    L = oracle.lib()
    x = np.linspace(lo, hi, 20001, dtype=np.float32)
    f = getattr(L, "gso_" + name)
    got = np.array([f(float(v)) for v in x], np.float32)
    exact = fn(x.astype(np.float64))
    assert ulp_err(got, exact) <= max_ulp


def test_atan2_accuracy_and_special_cases():
    L = oracle.lib()
    rng = np.random.Generator(np.random.PCG64(3))
    y = rng.normal(0, 10, 20000).astype(np.float32)
    x = rng.normal(0, 10, 20000).astype(np.float32)
    got = np.array([L.gso_atan2f(float(a), float(b)) for a, b in zip(y, x)], np.float32)
    exact = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert ulp_err(got, exact) <= 3.0
    inf = float("inf")
    for a, b in [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, 0.0),
                 (inf, inf), (-inf, -inf), (1.0, -inf), (0.0, 0.0), (-0.0, -0.0)]:
        assert L.gso_atan2f(a, b) == pytest.approx(float(np.float32(np.arctan2(a, b))), abs=1e-7)


def test_half_decoding_is_exact():
    L = oracle.lib()
    bits = np.arange(0, 65536, 7, dtype=np.uint32)
    ref = bits.astype(np.uint16).view(np.float16).astype(np.float32)
    got = np.array([L.gso_half_to_float(int(b)) for b in bits], np.float32)
    finite = np.isfinite(ref)
    assert np.array_equal(got[finite].view(np.uint32), ref[finite].view(np.uint32))


@pytest.fixture(scope="module")
def frame_result():
    scene = sc.uniform_cloud(6000, seed=77, log_scale=(-2.3, 0.7))
    frame = sc.make_frame(sc.look_at((1, 2, 11), (0, 0, 0)), 200, 120, 55.0, 0.1, 100.0,
                          raster_chunk_size=0)
    return scene, frame, oracle.render(scene, frame, 0)


def test_sorted_order_is_tile_depth_ordinal(frame_result):
    scene, frame, r = frame_result
    recs = r["sorted_records"]
    keys = r["proj_mean"][:, 2].view(np.uint32)
    order = np.lexsort((recs[:, 1], keys[recs[:, 1]], recs[:, 0]))
    assert np.array_equal(order, np.arange(recs.shape[0]))


def test_counts_match_emission_and_ranges(frame_result):
    scene, frame, r = frame_result
    recs = r["sorted_records"]
    assert recs.shape[0] == int(r["tile_counts"].sum()) == int(r["state"][1])
    per_gid = np.bincount(recs[:, 1], minlength=r["tile_counts"].size)
    assert np.array_equal(per_gid, r["tile_counts"])
    ntile = r["tiles_x"] * r["tiles_y"]
    assert np.all(recs[:, 0] < ntile)  # no sentinel padding needed
    off = r["tile_offsets"]
    assert np.array_equal(off, np.searchsorted(recs[:, 0], np.arange(ntile + 1), side="left"))
    assert np.all(np.diff(off.astype(np.int64)) >= 0)


def test_depth_sort_is_stable(frame_result):
    scene, frame, r = frame_result
    ds = r["depth_sorted"]
    assert np.all(np.diff(ds[:, 0].astype(np.int64)) >= 0)
    same = ds[1:, 0] == ds[:-1, 0]
    assert np.all(ds[1:, 1][same] > ds[:-1, 1][same])


def test_chunked_raster_matches_direct_when_transmittance_stays_high():
    scene = sc.uniform_cloud(4000, seed=5, log_scale=(-1.6, 0.3), opacity_logit=(-3.0, 0.5))
    base = sc.make_frame(sc.look_at((0, 0, 9), (0, 0, 0)), 64, 48, 60.0, 0.1, 100.0)
    direct = oracle.render(scene, dict(base, raster_chunk_size=0), 0)
    chunked = oracle.render(scene, dict(base, raster_chunk_size=256), 0)
    per_tile = np.diff(direct["tile_offsets"].astype(np.int64))
    assert per_tile.max() > 256  # the chunked path is exercised
    assert np.abs(direct["rgba"] - chunked["rgba"]).max() < 1e-4


def test_overflow_publishes_nothing():
    scene = sc.uniform_cloud(3000, seed=8, log_scale=(-2.0, 0.5))
    frame = sc.make_frame(sc.look_at((0, 0, 10), (0, 0, 0)), 96, 64, capacity=100, attempt=7,
                          last_version=3)
    sentinel = np.full((64, 96, 4), 0.25, np.float32)
    r = oracle.render(scene, frame, 0, rgba_init=sentinel)
    assert r["state"][3] == 1 and r["state"][0] == 0 and r["state"][1] > 100
    assert list(r["output_state"]) == [7, 3, int(r["state"][1]), 1]
    assert np.array_equal(r["rgba"], sentinel)
    ok = oracle.render(scene, dict(frame, capacity=10**8), 0)
    assert list(ok["output_state"])[:2] == [7, 7]


def test_fp32_restatement_close_to_fp64_twin(frame_result):
    scene, frame, r = frame_result
    r64 = oracle.render(scene, frame, 1)
    mse = float(np.mean((r["rgba"][..., :3] - r64["rgba"][..., :3]) ** 2))
    assert mse == 0 or 10 * np.log10(1.0 / mse) > 60
