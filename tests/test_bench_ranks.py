"""The multi-rank path of bench.py on CPU: replicas time independently and
the slowest one bounds the whole-job rate (gloo, world size 2); the
reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, value = bench.whole_job_rate([10.0, 30.0][rank], 5, world)
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_whole_job_rate_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            ms, value = out[r]
            assert ms == 30.0
            assert value == pytest.approx(2 * 5 / 0.030)


def test_single_rank_rate():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job_rate(20.0, 4, 1) == (20.0, pytest.approx(200.0))


def test_reference_arm_is_silent_off_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                        "q4_120x40", "--steps", "1", "--warmup", "1", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
