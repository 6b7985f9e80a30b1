"""Multi-process host logic of the replica bench path, on CPU (gloo, world size 2).

The path has no data exchange: every rank advances its own halos and the job's
throughput is the sum over ranks, timed by the slowest rank.  These tests run
the same helpers bench.py uses under torchrun, on gloo instead of NCCL.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 1.5 + r seconds for its 10 steps: the job takes the slowest
        el = bench.max_over_ranks(1.5 + rank, world)
        out[rank] = (el, bench.replica_throughput(10, world, el))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert set(out.keys()) == {0, 1}
    for r in range(world):
        el, value = out[r]
        assert el == pytest.approx(2.5)
        assert value == pytest.approx(10 * world / 2.5)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.replica_throughput(20, 1, 2.0) == 10.0


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_on_rank0_only(rank):
    """`bench.py --impl reference` under torchrun: rank 0 times the CPU path and
    prints one JSON line, the other ranks exit 0 without work."""
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--workload", "1", "--n", "16", "--steps", "2", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if rank == 0:
        assert len(lines) == 1
        d = json.loads(lines[0])
        assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
        assert d["cpu_baseline"]["kind"] == "port"
    else:
        assert lines == []


def test_gpus_flag_launches_one_process_per_rank():
    """`bench.py --gpus 2` started as one process spawns its two ranks itself (as
    torchrun would): exactly one JSON line comes back, from rank 0, and it
    reports two GPUs.  The reference arm needs no GPU, so this runs on CPU."""
    pytest.importorskip("torch")
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR",
                                                           "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--workload", "1", "--n", "16", "--steps", "2", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2


def test_world_size_must_match_gpus_flag():
    env = dict(os.environ, RANK="0", WORLD_SIZE="2", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "4",
                        "--workload", "1", "--n", "16", "--steps", "1", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and "WORLD_SIZE=2" in r.stderr
