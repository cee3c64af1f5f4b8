"""bench.py's replica logic at world size 2 on CPU (gloo): the barrier and
maximum of the per-rank times, the whole-job throughput, and the reference
arm's rank filter (only rank 0 runs and prints).  No GPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    local_s = 1.0 + rank  # rank 1 is the slower one
    t = bench.ranks_max(local_s, dist, device="cpu")
    v = bench.replica_gups(10 ** 9, world, t)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, v))


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]          # both ranks see the max time
    assert [r[2] for r in res] == [1.0, 1.0]          # 2 ranks x 1e9 updates / 2 s = 1 GUPS


def test_ranks_max_without_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.ranks_max(3.5, None) == 3.5
    assert bench.replica_gups(2 * 10 ** 9, 1, 2.0) == 1.0


def test_reference_arm_only_rank0_prints():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
