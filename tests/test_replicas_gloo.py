"""Replica path of bench.py on CPU (world size 2, gloo on 127.0.0.1): the
pass does not shard (frames and requests are independent), so N GPUs run N
replicas; the job's time is the slowest rank's and its throughput counts
every rank's frames."""
import importlib.util
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    b = _bench()
    ms = [12.5, 17.25][rank]  # per-rank device time of the same step count
    slowest = b.max_over_ranks(ms, world, device="cpu")
    fps = b.job_frames_per_s(10, 16, world, slowest / 1000.0)
    dist.barrier()
    out[rank] = (slowest, fps)
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_count_every_rank():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0] == out[1]
    slowest, fps = out[0]
    assert slowest == 17.25
    assert fps == pytest.approx(10 * 16 * 2 / 0.01725)


def test_single_rank_needs_no_process_group():
    b = _bench()
    assert b.max_over_ranks(3.0, 1) == 3.0
    assert b.job_frames_per_s(2, 16, 1, 0.5) == 64.0
