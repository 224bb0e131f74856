"""bench.py host logic (no GPU): the multi-rank reduction over gloo ranks
and the JSON line of the reference arm."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, times, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.job_time_ms(times[rank], dist, torch, "cpu")
        value = bench.job_throughput(world, 1000, 10, ms)
        out.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_job_time_is_max_over_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [12.5, 20.0]
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q))
             for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in got:
        assert ms == 20.0
        # two replicas of 1000 bonds, 10 steps, in 20 ms
        assert value == pytest.approx(2 * 1000 * 10 / 0.020)


def test_single_rank_time_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_time_ms(3.0, None, None, "cpu") == 3.0


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--gpus", "2", "--steps",
                          "1", "--warmup", "0"], env=env, capture_output=True,
                         text=True, timeout=300)
    assert res.returncode == 0
    assert res.stdout.strip() == ""


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle",
                                                    "libpp_oracle.so")),
                    reason="oracle not built")
def test_reference_arm_line():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--steps", "1", "--warmup",
                          "0"], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "bond-updates/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
