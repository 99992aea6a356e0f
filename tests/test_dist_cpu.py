"""The N > 1 path of the benchmark on CPU: two gloo ranks on 127.0.0.1.

The path does not shard (one resident partition per GPU): N GPUs run N
independent replicas, and the whole-job value is all ranks' units over the
slowest rank's time.  The reference arm runs on rank 0 only.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took 1 + r seconds for the same 1000 units
    v = bench.whole_job_rate(1000, 1.0 + rank, world)
    t = bench.max_over_ranks(0.5 * (rank + 1), world)
    dist.destroy_process_group()
    out.put((rank, v, t))


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # 2 ranks x 1000 units over the slowest rank's 2 s, on every rank
    assert [v for _, v, _ in res] == [1000.0, 1000.0]
    assert [t for _, _, t in res] == [1.0, 1.0]


def test_reference_arm_is_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
