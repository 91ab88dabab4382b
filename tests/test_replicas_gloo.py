"""The N > 1 replica path of bench.py on CPU, with two gloo ranks: the step time is
the maximum over ranks and the whole-job rate counts every rank's GEMMs; the
reference arm runs on rank 0 only."""
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


def worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.reduce_max(1.0 + rank * 0.25, world)  # rank 1 is the slow one
        q.put((rank, t, bench.replica_gops(2048, 4096, 2048, t * 1e-3, world)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_replica_rate_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t, rate in got:
        assert t == 1.25  # every rank sees the slowest rank's time
        assert rate == pytest.approx(2 * 2.0 * 2048 * 4096 * 2048 / 1.25e-3 / 1e9)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.replica_gops(10, 20, 30, 1.0, 1) == pytest.approx(2.0 * 10 * 20 * 30 / 1e9)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == ""
