#!/usr/bin/env python3
"""Benchmark of the tiled Gaussian-splatting pass on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): 3,000,000
Gaussians from a 64-cluster anisotropic mixture in the reference's compact
layout (f16 log-scales/opacity, oct101012 rotation, rgb8e8 SH degree 3),
rendered at 1920x1080 from 16 seeded cameras on a radius-30 orbit. A step is
one pass over all 16 cameras (16 frames). Inputs are synthetic (seeded), the
scene (288 MB of packed buffers) is resident in HBM and larger than L2.

Prints one JSON line. ``--impl reference`` times the CPU restatement of the
reference's pass (the oracle: the reference itself is WGSL/TSL for a browser
WebGPU device, which is unavailable here) on the host cores instead.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "3dgs_tile_webgpu_gb300"
METRIC = "frames/s @1080p, 3M splats: batched fp16 vs plain fp32 (PSNR≥50dB); p99 ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--splats", type=int, default=3_000_000)
    ap.add_argument("--cameras", type=int, default=16)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--precision", default="half2", choices=["fp32", "exact", "half2"],
                    help="raster form of the batched (headline) measurement: the metric's batched fp16 is half2")
    ap.add_argument("--plain-precision", default="fp32", choices=["fp32", "exact"])
    ap.add_argument("--latency-frames", type=int, default=240)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape for the batched form")
    ap.add_argument("--views-per-launch", type=int, default=None,
                    help="fixed launch shape for the batched form instead of the autotuner's")
    ap.add_argument("--tile-size", type=int, default=None, choices=[8, 16, 32],
                    help="fixed tile size for the batched form instead of the autotuner's")
    ap.add_argument("--pixels-per-lane", type=int, default=None, choices=[2, 4],
                    help="fixed raster block shape for the batched form instead of the autotuner's")
    ap.add_argument("--forms", default="all", choices=["all", "batched"],
                    help="'batched' skips the timed plain (one view per launch) form")
    ap.add_argument("--serve", action="store_true", help="serving-loop measurement (configuration 4)")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip configurations 3, 5 and 4 after the headline workload")
    ap.add_argument("--config3", action="store_true",
                    help="multi-cloud, multi-view batch (configuration 3): 8 clouds, 32 mixed-resolution cameras")
    ap.add_argument("--config5", action="store_true",
                    help="configuration 5: 12M far-origin splats at 3840x2160, FP64 projection form")
    ap.add_argument("--serve-rates", default="200,500,1000,2000")
    ap.add_argument("--serve-concurrency", type=int, default=64,
                    help="closed-loop measurement: requests kept outstanding (0 skips it)")
    ap.add_argument("--serve-lanes", type=int, default=2)
    ap.add_argument("--serve-max-views", type=int, default=16)
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-scale", type=float, default=1.0, help="scales the resident scene sizes")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


PROFILES = os.path.join(ROOT, "profiles")


def measured_traffic_per_view(stage: str, args) -> int | None:
    """DRAM bytes (read + write) per view of `stage`'s kernel, from a
    committed ncu summary taken on a smaller batch of this scene and
    resolution (the traffic grows in proportion to the views)."""
    try:
        names = sorted(f for f in os.listdir(PROFILES) if f.endswith(".md"))
    except OSError:
        return None
    for name in names:
        with open(os.path.join(PROFILES, name)) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 7 and parts[0] == "traffic_per_view" and parts[1] == stage:
                    try:
                        cfg = (int(parts[2]), int(parts[3]), int(parts[4]), parts[5])
                        if cfg == (args.splats, args.width, args.height, args.precision):
                            return int(parts[6])
                    except ValueError:
                        continue
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def stage_bytes(stage: str, n: int, v: int, inter: int, tiles: int, pixels: int, coeffs: int, depth_passes: int,
                tile_passes: int, color_bytes: int, depth_out: bool, groups: int = 1, precision: str = "half2",
                views: int = 1) -> int:
    """Algorithmic DRAM bytes of each stage over one batch (the data it must move).

    n, v, inter, tiles, pixels: totals over the batch's `views` views (all of
    one scene); groups: view groups (the views of one launch share one read of
    the packed scene); precision: raster form (half2 reads the 32-byte packed record per
    intersection, fp32 that record plus the FP32 colour, exact the reference's
    mean, conic and colour)."""
    fast = precision != "exact"
    if stage == "project":
        # Read once per group: the tail, mean + id, shape and rotation of every
        # splat, the SH of every splat visible in some view of the group.
        n_scene, per_group = n // max(1, views), max(1, views // max(1, groups))
        sh = min(n_scene, (v // max(1, views)) * per_group) * 4 * coeffs
        scene = groups * (n_scene * (4 + 16 + 8 + 4) + sh)
        # Written per view: mean, count, key of every item; conic, colour and
        # the emission (and, fast forms, raster) record of every visible one.
        written = n * (16 + 4 + 4) + v * (16 + 16 + 32 + (32 if fast else 0))
        return scene + written
    if stage == "compact":
        return n * 4 + n * 4 + v * 8
    if stage == "depth_sort":
        return depth_passes * v * 16
    if stage == "scan":
        return v * (4 + 4) + v * 8
    if stage == "emit":
        return v * (4 + 32 + 4 + 4) + inter * 8
    if stage == "tile_sort":
        return tile_passes * inter * 16
    if stage == "ranges":
        return inter * 4 + (tiles + 1) * 4
    if stage == "raster":
        per_record = 32 if precision == "half2" else 48
        return (tiles + 1) * 4 + inter * (4 + per_record) + pixels * (color_bytes + (4 if depth_out else 0))
    return 0


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's value (replicas: the job ends with its last rank)."""
    if world <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_frames_per_s(steps: int, frames_per_step: int, world: int, seconds: float) -> float:
    """Whole-job throughput: every replica renders its own frames_per_step
    frames per step (weak scaling), timed by the slowest rank."""
    return steps * frames_per_step * world / seconds


def run_reference(args) -> None:
    """CPU restatement of the pass (the oracle) on all host threads."""
    world, rank, _ = dist()
    if rank != 0:
        return
    import oracle
    sc = importlib.import_module(PKG + ".scenes")
    scene = sc.clustered_cloud(args.splats, seed=1002)
    frames = sc.config2_frames(args.cameras, args.width, args.height)
    cores = oracle.lib().gso_num_threads()
    for i in range(args.warmup):
        oracle.render(scene, frames[i % len(frames)], 0, output_depth=False)
    t0 = time.perf_counter()
    for i in range(args.steps):
        oracle.render(scene, frames[i % len(frames)], 0, output_depth=False)
    dt = time.perf_counter() - t0
    fps = args.steps / dt
    out = {
        "metric": METRIC, "value": fps, "unit": "frames/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{args.splats} clustered Gaussians, {args.width}x{args.height}, "
                               f"{args.cameras} orbit cameras (one frame per step)",
                   "splats": args.splats, "width": args.width, "height": args.height, "cameras": args.cameras},
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": "one 1080p frame of the 3M-splat scene per step (FP32 restatement, OpenMP)"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_serving(args) -> None:
    print(json.dumps(serving_result(args)))


def serving_result(args) -> dict:
    """Configuration 4: four resident scenes (0.5M, 1.5M, 3M, 6M Gaussians,
    configuration-1 distributions), Poisson arrivals, a random orbit camera
    and a size from {720p, 1080p, 1440p} per request, 40 GB workspace budget,
    half2 blending with FP32 accumulation."""
    import numpy as np
    import torch
    sc = importlib.import_module(PKG + ".scenes")
    dev = importlib.import_module(PKG + ".device")
    srv = importlib.import_module(PKG + ".serving")
    importlib.import_module(PKG).load()
    sizes = {"0.5M": 500_000, "1.5M": 1_500_000, "3M": 3_000_000, "6M": 6_000_000}
    scenes = {k: dev.DeviceScene(sc.uniform_cloud(max(1000, int(n * args.serve_scale)), seed=1004 + i,
                                                  extent=5.0 * (n / 1e5) ** (1 / 3)))
              for i, (k, n) in enumerate(sizes.items())}
    res = [(1280, 720), (1920, 1080), (2560, 1440)]
    rng = np.random.Generator(np.random.PCG64(1004))

    def frame_for(name, w, h):
        radius = 15.0 * (sizes[name] / 1e5) ** (1 / 3)
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(-0.5, 0.5)
        eye = radius * np.array([np.cos(el) * np.sin(az), np.sin(el), np.cos(el) * np.cos(az)])
        return sc.make_frame(sc.look_at(eye, (0, 0, 0)), w, h, 60.0, 0.1, 1000.0)

    server = srv.RenderServer(scenes, lanes=args.serve_lanes, budget_bytes=40e9, max_views=args.serve_max_views,
                              precision="half2")
    server.probe({(k, w, h): frame_for(k, w, h) for k in scenes for (w, h) in res})
    results = {}
    closed = None
    if args.serve_concurrency > 0:
        # Closed loop: `concurrency` requests always outstanding; each
        # completion is replaced by a new request at once.
        def make_request(i):
            name = list(scenes)[int(rng.integers(0, len(scenes)))]
            w, h = res[int(rng.integers(0, len(res)))]
            return srv.Request(i, name, frame_for(name, w, h))
        torch.cuda.synchronize()
        closed = server.run_closed(make_request, args.serve_concurrency, args.serve_requests * 2,
                                   warmup=args.serve_concurrency)
        closed["target_p99_ms"] = 10.0
        closed["target_met"] = closed["p99_ms"] is not None and closed["p99_ms"] < 10.0
    for rate in [float(r) for r in args.serve_rates.split(",") if r]:
        server.completed = []
        server.batches = server.retries = 0
        t, reqs = 0.0, []
        for i in range(args.serve_requests):
            t += rng.exponential(1.0 / rate)
            name = list(scenes)[int(rng.integers(0, len(scenes)))]
            w, h = res[int(rng.integers(0, len(res)))]
            reqs.append(srv.Request(i, name, frame_for(name, w, h), arrival=t))
        torch.cuda.synchronize()
        results[str(int(rate))] = server.run(reqs)
    server.close()
    best = max(list(results.values()) + ([closed] if closed else []), key=lambda r: r["frames_per_s"])
    return {
        "metric": "serving: p50/p99 ms and frames/s at Poisson request rates (configuration 4)",
        "value": best["frames_per_s"], "unit": "frames/s", "n_gpus": 1, "higher_is_better": True,
        "dtype": "f16", "data": "synthetic",
        "config": {"workload": "4 resident scenes (0.5M/1.5M/3M/6M), 720p/1080p/1440p, orbit cameras, "
                               f"40 GB workspace budget, {args.serve_lanes} lanes, "
                               f"<= {args.serve_max_views} views per batch",
                   "scene_scale": args.serve_scale, "requests_per_rate": args.serve_requests,
                   "lanes": args.serve_lanes, "max_views": args.serve_max_views},
        "rates": results,
        "closed_loop": closed,
    }


def run_config3(args) -> None:
    print(json.dumps(config3_result(args)))


def config3_result(args) -> dict:
    """Configuration 3: one store of 8 transformed clouds (50k..2M splats),
    32 cameras at 640x480..3840x2160, all views in one graph-captured batch
    with the autotuned launch shape; half2 raster."""
    import numpy as np
    import torch
    P = importlib.import_module(PKG)
    sc = importlib.import_module(PKG + ".scenes")
    dev = importlib.import_module(PKG + ".device")
    P.load()
    scene, worlds = sc.config3_scene()
    frames = sc.config3_frames(worlds, 32)
    ds = dev.DeviceScene(scene)
    data = ds.data()
    colors = [torch.empty((f["height"], f["width"], 4), dtype=torch.float16, device="cuda") for f in frames]
    cams = [P.make_camera(f) for f in frames]
    views = [(data, c, f["width"], f["height"], colors[i].data_ptr(), 0, "rgba16f")
             for i, (c, f) in enumerate(zip(cams, frames))]
    pipe = P.TiledGaussianPipeline(data, {"raster_precision": args.precision, "intersection_capacity": 1 << 26})
    while True:  # grow the intersection workspace until the whole batch fits (capacity policy headroom 1.25)
        pipe.render_batch(views)
        st = pipe.read_stats()
        if not st["overflow"]:
            break
        pipe.resize_intersections(int(st["requestedIntersections"] * 1.25) + 256)
    tune_ms = None
    if not args.no_autotune:
        _, tune_ms = pipe.autotune(views, trials=2)
    tuning = pipe.get_tuning()
    pipe.render_batch(views)
    stats = pipe.read_stats()
    stream = torch.cuda.Stream()
    pipe.capture_graph(views, stream.cuda_stream)
    for _ in range(max(args.warmup, 3)):
        with torch.cuda.stream(stream):
            pipe.launch_graph(cams, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            pipe.launch_graph(cams, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    psnr_db = None
    if not args.no_cpu_baseline:
        import oracle
        small = min(range(len(frames)), key=lambda i: frames[i]["width"] * frames[i]["height"])
        img = colors[small].float().cpu().numpy()
        o64 = oracle.render(scene, frames[small], 1, output_depth=False)
        mse = float(np.mean((img[..., :3].astype(np.float64) - o64["rgba"][..., :3]) ** 2))
        psnr_db = float("inf") if mse == 0 else 10 * np.log10(1.0 / mse)
    pixels = sum(f["width"] * f["height"] for f in frames)
    pipe.dispose()
    return {
        "metric": "frames/s, configuration 3 (8 clouds, 32 mixed-resolution cameras, one graph-captured batch)",
        "value": len(frames) / (ms / 1000.0), "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f16", "data": "synthetic",
        "config": {"workload": f"{scene['count']} Gaussians in 8 objects (50k..2M, rigid + scale U(0.5,2)), "
                               f"32 cameras, resolutions 640x480..3840x2160 ({pixels / 1e6:.1f} MPix per batch)",
                   "launch_shape": tuning, "autotune_ms_per_batch": tune_ms},
        "stats": {"visible": stats["visibleGaussianCount"], "intersections": stats["intersectionCount"]},
        "megapixels_per_s": pixels / 1e6 / (ms / 1000.0),
        "psnr_db_vs_fp64_smallest_view": psnr_db, "clocks": ck,
    }


def run_config5(args) -> None:
    print(json.dumps(config5_result(args)))


def config5_result(args) -> dict:
    """Configuration 5: 12M splats in clusters centred at (1e5, 1e5, 0) with 5%
    near-degenerate axes, one 3840x2160 view, FP64 projection form (far-origin
    mean transform and near-singular conic in double) and the half2 raster;
    about 3.9e8 intersections, past the reference's own record cap, so the
    parity is the oracle's (tests/test_gpu_precision.py)."""
    import numpy as np
    import torch
    P = importlib.import_module(PKG)
    dev = importlib.import_module(PKG + ".device")
    sc = importlib.import_module(PKG + ".scenes")
    far = (1e5, 1e5, 0.0)
    scene = sc.clustered_cloud(12_000_000, seed=1005, offset=far, log_scale=(-2.0, 1.0), degenerate_fraction=0.05)
    eye = np.array(far) + np.array([0.0, 5.0, 30.0])
    frame = sc.make_frame(sc.look_at(eye, far), 3840, 2160, 60.0, 0.1, 1000.0)
    ds = dev.DeviceScene(scene)
    W, H = 3840, 2160
    color = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    pipe = P.TiledGaussianPipeline(ds.data(), {"raster_precision": args.precision, "projection_precision": "fp64",
                                               "intersection_capacity": 1 << 26})
    pipe.prepare_frame(W, H)
    cam = P.make_camera(frame)
    while True:  # grow the intersection workspace until the frame fits (capacity policy headroom 1.25)
        pipe.render(cam, color.data_ptr(), 0, color_format="rgba16f")
        st = pipe.read_stats()
        if not st["overflow"]:
            break
        pipe.resize_intersections(int(st["requestedIntersections"] * 1.25) + 256)
    for _ in range(max(args.warmup, 3)):
        pipe.render(cam, color.data_ptr(), 0, color_format="rgba16f")
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        pipe.render(cam, color.data_ptr(), 0, color_format="rgba16f")
    e1.record()
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    st = pipe.read_stats()
    pipe.dispose()
    return {
        "metric": "frames/s, configuration 5 (12M far-origin splats, 3840x2160, FP64 projection form)",
        "value": 1000.0 / ms, "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "dtype": "f16" if args.precision == "half2" else "f32",
        "data": "synthetic",
        "config": {"workload": "12000000 Gaussians, 64 clusters centred at (1e5, 1e5, 0), log-scales N(-2, 1), "
                               "5% near-degenerate axes, 3840x2160, FP64 projection form"},
        "stats": {"visible": st["visibleGaussianCount"], "intersections": st["intersectionCount"]},
        "intersections_per_s": st["intersectionCount"] / (ms / 1000.0), "clocks": ck,
    }


def main() -> None:
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.serve:
        run_serving(args)
        return
    if args.config3:
        run_config3(args)
        return
    if args.config5:
        run_config5(args)
        return
    import numpy as np
    import torch

    world, rank, local = dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    P = importlib.import_module(PKG)
    sc = importlib.import_module(PKG + ".scenes")
    dev = importlib.import_module(PKG + ".device")
    P.load()
    scene = sc.clustered_cloud(args.splats, seed=1002)
    frames = sc.config2_frames(args.cameras, args.width, args.height)
    cams = [P.make_camera(f) for f in frames]
    ds = dev.DeviceScene(scene)
    W, H = args.width, args.height
    ncam = len(cams)

    def make_pipe(precision):
        pp = P.TiledGaussianPipeline(ds.data(), {"raster_precision": precision, "intersection_capacity": 1 << 26})
        pp.prepare_frame(W, H)
        return pp

    plain = make_pipe(args.plain_precision)
    colors = [torch.empty((H, W, 4), dtype=torch.float16, device="cuda") for _ in range(ncam)]
    host = [torch.empty((H, W, 4), dtype=torch.float16, pin_memory=True) for _ in range(ncam)]
    data = ds.data()

    # Size the intersection workspace from the demand of every camera
    # (IntersectionCapacityPolicy headroom 1.25).
    demand, stats = 0, []
    for cam in cams:
        plain.render(cam, colors[0].data_ptr(), 0, color_format="rgba16f")
        st = plain.read_stats()
        stats.append(st)
        demand = max(demand, st["requestedIntersections"])
    plain.resize_intersections(int(demand * 1.25) + 256)

    def step_plain():
        launches = 0
        for i, cam in enumerate(cams):
            plain.render(cam, colors[i].data_ptr(), 0, color_format="rgba16f")
            launches += plain.last_launch_count()
        return launches

    def timed(step, pipe_for_stages, stream_for_timing=None):
        """Device time of exactly `steps` steps (no instrumentation), then the
        per-stage breakdown from a second, profiled run of as many steps."""
        stream_for_timing = stream_for_timing or torch.cuda.current_stream()
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        clocks = Clocks(local)
        barrier()
        torch.cuda.synchronize()
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream_for_timing)
        nl = 0
        for _ in range(args.steps):
            nl += step()
        e1.record(stream_for_timing)
        torch.cuda.synchronize()
        ck = clocks.stop()
        barrier()
        ms = e0.elapsed_time(e1)
        sm, prof = {}, 0
        if pipe_for_stages is not None:
            pipe_for_stages.set_profiling(True)
            pipe_for_stages.stage_times()
            for _ in range(args.steps):
                step()
            torch.cuda.synchronize()
            sm, prof = pipe_for_stages.stage_times()
            pipe_for_stages.set_profiling(False)
        ms = max_over_ranks(ms, world)
        return ms, sm, prof, nl, ck

    fps_plain = stage_ms_plain = launches_plain = clocks_plain = None
    if args.forms == "all":
        ms_plain, stage_ms_plain, prof_plain, launches_plain, clocks_plain = timed(step_plain, plain)
        fps_plain = job_frames_per_s(args.steps, ncam, world, ms_plain / 1000.0)

    # Batched form: all cameras of a step in one launch sequence.
    batched = P.TiledGaussianPipeline(ds.data(), {"raster_precision": args.precision,
                                                  "intersection_capacity": int(demand * 1.25 * ncam) + 256})
    views = [(data, cam, W, H, colors[i].data_ptr(), 0, "rgba16f") for i, cam in enumerate(cams)]
    gstream = torch.cuda.Stream()
    # Launch shape from the autotuner (outputs do not depend on it), before
    # the untimed sizing render and the graph capture.
    tune_ms = None
    if args.views_per_launch is not None:
        batched.set_tuning({"views_per_launch": args.views_per_launch})
    elif not args.no_autotune:
        _, tune_ms = batched.autotune(views, trials=3)
    if args.tile_size is not None:
        batched.set_tuning({"tile_size": args.tile_size})
    if args.pixels_per_lane is not None:
        batched.set_tuning({"raster_pixels_per_lane": args.pixels_per_lane})
    tuning = batched.get_tuning()
    batched.render_batch(views)  # size the workspaces, then capture the pass as a graph
    torch.cuda.synchronize()
    batched.capture_graph(views, gstream.cuda_stream)

    def step_batched():
        batched.render_batch(views)
        return batched.last_launch_count()

    def step_graph():
        with torch.cuda.stream(gstream):
            batched.launch_graph(cams, stream=gstream.cuda_stream)
        return batched.last_launch_count()

    # Direct batches (one render_batch call per step), then the per-stage
    # breakdown from a profiled run of as many steps.
    ms_direct, stage_ms, profiled, launches_direct, clock_direct = timed(step_batched, batched)
    # Stage times are means per launch sequence; a batch may run as several.
    seq_per_batch = profiled / args.steps if profiled else 1.0
    stage_ms = {k: v * seq_per_batch for k, v in stage_ms.items()}
    fps_direct = job_frames_per_s(args.steps, ncam, world, ms_direct / 1000.0)
    # The headline: the same batches replayed from the captured graph (one
    # graph launch per step; each replay restages the cameras).
    ms_total, _, _, launches, clock_info = timed(step_graph, None, gstream)
    fps = job_frames_per_s(args.steps, ncam, world, ms_total / 1000.0)
    fps_graph = fps
    bstats = batched.read_stats()

    # Latency distributions: one frame (plain) and one 16-camera batch, each
    # synchronised on its own.
    def latencies(fn, count):
        out = []
        for i in range(count):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn(i)
            b.record()
            b.synchronize()
            out.append(a.elapsed_time(b))
        out.sort()
        return out[len(out) // 2], out[min(len(out) - 1, int(0.99 * len(out)))]

    p50_plain = p99_plain = None
    if args.forms == "all":
        p50_plain, p99_plain = latencies(lambda i: plain.render(cams[i % ncam], colors[0].data_ptr(), 0,
                                                                color_format="rgba16f"), args.latency_frames)
    def batch_once(i):
        with torch.cuda.stream(gstream):
            batched.launch_graph(cams, stream=gstream.cuda_stream)

    p50, p99 = latencies(batch_once, max(20, args.latency_frames // ncam))

    # End to end through the public API (batched form): camera/object tables
    # from host memory in, every rendered rgba16f image back to pinned host
    # memory, every step. Two pipelines with their own targets alternate, so
    # the read-back of step k (on a copy stream) overlaps the render of step
    # k + 1; a pipeline renders again only after its previous images are back.
    colors2 = [torch.empty_like(c) for c in colors]
    batched2 = P.TiledGaussianPipeline(ds.data(), {"raster_precision": args.precision,
                                                   "intersection_capacity": int(demand * 1.25 * ncam) + 256})
    batched2.set_tuning(tuning)
    views2 = [(data, cam, W, H, colors2[i].data_ptr(), 0, "rgba16f") for i, cam in enumerate(cams)]
    gstream2 = torch.cuda.Stream()
    batched2.render_batch(views2)
    torch.cuda.synchronize()
    batched2.capture_graph(views2, gstream2.cuda_stream)
    lanes = [(batched, gstream, colors), (batched2, gstream2, colors2)]
    copy_stream = torch.cuda.Stream()
    copied = [None, None]  # event: lane's images are back in host memory
    rendered = [None]      # event: the previous step's render finished

    def e2e_step(k):
        # Renders run one after another (each pass expects the whole GPU);
        # only the read-back overlaps the next render.
        pipe, gs, targets = lanes[k & 1]
        with torch.cuda.stream(gs):
            if copied[k & 1] is not None:
                gs.wait_event(copied[k & 1])
            if rendered[0] is not None:
                gs.wait_event(rendered[0])
            pipe.launch_graph(cams, stream=gs.cuda_stream)
            done = torch.cuda.Event()
            done.record(gs)
            rendered[0] = done
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(done)
            for hb, c in zip(host, targets):
                hb.copy_(c, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(copy_stream)
            copied[k & 1] = ev

    for k in range(2):
        e2e_step(k)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)
    frames_done = args.steps * ncam * world
    e2e_fps = frames_done / e2e_s
    h2d = ncam * (16 * 4 + 40 * 4)  # projection + one object row per view
    d2h = ncam * W * H * 8

    # Roofline of every stage; the dominant one is reported as `roofline`.
    hbm, peak_kind = peaks()
    mean_stats = {k: statistics.mean(s[k] for s in stats) for k in ("visibleGaussianCount", "requestedIntersections")}
    n, v, inter = scene["active_count"], int(mean_stats["visibleGaussianCount"]), int(mean_stats["requestedIntersections"])
    tile_px = int(tuning.get("tile_size", 16))
    tiles = ((W + tile_px - 1) // tile_px) * ((H + tile_px - 1) // tile_px)
    stages = {}
    # per batch: every stage processes all views of the step, in launches of
    # views_per_launch views (one view group each: the views share the scene);
    # visible and intersection totals are the batched pass's own (its tile
    # size sets the intersections)
    bn, bv_, bi, bt = n * ncam, int(bstats["visibleGaussianCount"]), int(bstats["intersectionCount"]), tiles * ncam
    vpl = int(tuning["views_per_launch"]) or ncam
    nlaunch = (ncam + vpl - 1) // vpl
    ltile_bits = max(1, int(np.ceil(np.log2(tiles * min(vpl, ncam) + 1))))
    btile_passes = min(4, (ltile_bits + int(tuning["tile_digit_bits"]) - 1) // int(tuning["tile_digit_bits"]))
    for name, ms in stage_ms.items():
        b = stage_bytes(name, bn, bv_, bi, bt, W * H * ncam, 16, 4, btile_passes, 8, False, groups=nlaunch,
                        precision=args.precision, views=ncam)
        gbs = b / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        stages[name] = {"ms": ms, "bytes": b, "GB/s": gbs, "frac": gbs / hbm}
    dom = max(stages, key=lambda k: stages[k]["ms"])

    # The raster's own bound is FP32 arithmetic, not HBM: FLOPs = 12 checked
    # + 10 blended samples (the reference's rasterStats counters,
    # TileRasterizer.ts:545-546,617,702), counted in an untimed pass of the
    # same batch with the counters on, over the raster's CUDA-event time,
    # against SMs x 128 FP32 lanes x 2 x the median SM clock sampled during
    # the timed steps (MEASURED_PEAKS.json carries no FP32 figure).
    counting = P.TiledGaussianPipeline(ds.data(), {"raster_precision": args.precision, "raster_stats": True,
                                                   "intersection_capacity": int(demand * 1.25 * ncam) + 256})
    counting.set_tuning(tuning)
    counting.render_batch(views)
    work = counting.read_stats()["rasterWork"]
    counting.dispose()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    clock_mhz = clock_info.get("sm_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * clock_mhz * 1e6 / 1e12  # TFLOP/s
    raster_flops = 12 * work["checked"] + 10 * work["blended"]
    raster_s = stage_ms["raster"] * 1e-3
    raster_tflops = raster_flops / raster_s / 1e12 if raster_s > 0 else 0.0
    raster_fp32 = {"kernel": "raster", "bound": "fp32", "achieved": raster_tflops, "peak": fp32_peak,
                   "unit": "TFLOP/s", "frac": raster_tflops / fp32_peak,
                   "flops_per_batch": raster_flops, "checked": work["checked"], "blended": work["blended"],
                   "exp_per_s": work["blended"] / raster_s if raster_s > 0 else 0.0,
                   "peak_source": f"{sms} SMs x 128 FP32 lanes x 2 x {clock_mhz:.0f} MHz (median sampled SM clock)"}
    per_view = measured_traffic_per_view(dom, args) if tile_px == 16 else None
    traffic_per_launch = per_view * min(vpl, ncam) if per_view else None
    if dom == "raster":
        roofline = dict(raster_fp32, traffic=traffic_per_launch,
                        algorithmic_bytes_per_launch=stages[dom]["bytes"] / nlaunch,
                        traffic_unit="DRAM bytes per launch (ncu, scaled from a 4-view capture)",
                        hbm={"achieved": stages[dom]["GB/s"], "peak": hbm, "unit": "GB/s",
                             "frac": stages[dom]["frac"], "bytes_per_batch": stages[dom]["bytes"],
                             "peak_source": peak_kind})
    else:
        roofline = {"kernel": dom, "bound": "hbm", "achieved": stages[dom]["GB/s"], "peak": hbm, "unit": "GB/s",
                    "frac": stages[dom]["frac"], "traffic": traffic_per_launch,
                    "traffic_unit": "DRAM bytes per launch (ncu)", "peak_source": peak_kind}

    # Image quality of camera 0 against the FP64 oracle, and the CPU baseline.
    cpu = None
    psnr_db = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        batched.render_batch(views)
        torch.cuda.synchronize()
        img = colors[0].float().cpu().numpy()
        t0 = time.perf_counter()
        o32 = oracle.render(scene, frames[0], 0, output_depth=False)
        cpu_s = time.perf_counter() - t0
        o64 = oracle.render(scene, frames[0], 1, output_depth=False)
        mse = float(np.mean((img[..., :3].astype(np.float64) - o64["rgba"][..., :3]) ** 2))
        psnr_db = float("inf") if mse == 0 else 10 * np.log10(1.0 / mse)
        cpu = {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": oracle.lib().gso_num_threads(), "kind": "port",
               "sample": "camera 0 of the workload, one 1080p frame (FP32 restatement, OpenMP)"}

    plain.dispose()
    batched.dispose()
    batched2.dispose()
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16" if args.precision == "half2" else "f32", "data": "synthetic",
        "config": {"workload": f"{args.splats} clustered Gaussians (64-cluster mixture, SH3 rgb8e8, compact), "
                               f"{W}x{H}, {len(cams)} orbit cameras per step rendered as one batch "
                               f"replayed from a captured CUDA graph, {args.precision} raster",
                   "splats": args.splats, "width": W, "height": H, "cameras": len(cams),
                   "frames_per_step": len(cams), "parallelism": f"replicas x{world}",
                   "launch_shape": tuning,
                   "l2": "inputs larger than L2 (288 MB packed scene read every frame)",
                   "visible_mean": v, "intersections_mean": inter,
                   "batched_intersections_per_view": int(bstats["intersectionCount"]) // ncam},
        "p50_ms": p50, "p99_ms": p99, "psnr_db_vs_fp64": psnr_db,
        "forms": {"batched": {"precision": args.precision, "frames_per_s": fps, "views_per_batch": ncam,
                              "tuning": tuning, "autotune_ms_per_batch": tune_ms,
                              "graph_replay_frames_per_s": fps_graph,
                              "direct_frames_per_s": fps_direct, "direct_clocks": clock_direct,
                              "direct_gpu_launches": launches_direct,
                              "p50_batch_ms": p50, "p99_batch_ms": p99, "psnr_db": psnr_db,
                              "stats": bstats},
                  "plain": {"precision": args.plain_precision, "frames_per_s": fps_plain,
                            "p50_ms": p50_plain, "p99_ms": p99_plain, "stages_ms": stage_ms_plain,
                            "gpu_launches": launches_plain, "clocks": clocks_plain}},
        "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roofline,
        "raster_fp32": raster_fp32,
        "stages": stages,
        "profiled_renders": profiled,
        "clocks": clock_info,
        "cpu_baseline": cpu,
    }
    if world == 1 and args.forms == "all" and not args.no_other_configs:
        # The other benchmark configurations, measured in the same run (each
        # with its own resident scene and pipeline, after this workload's
        # pipelines are released): configuration 3 (batching), 5 (FP64
        # projection form) and 4 (serving).
        out["other_configs"] = {}
        for name, fn in (("config3", config3_result), ("config5", config5_result), ("serving", serving_result)):
            try:
                out["other_configs"][name] = fn(args)
            except Exception as exc:  # reported in the line; the headline stands
                out["other_configs"][name] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
