"""The N > 1 path of bench.py on CPU: two gloo ranks each time a replica,
the job's time is the slowest rank's and the rate counts every rank's work;
the reference arm does its work on rank 0 only."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    elapsed = [40.0, 55.0][rank]
    slowest = bench.max_over_ranks(elapsed, world)
    rate = bench.whole_job_rate(256, world, 10, slowest)
    dist.barrier()
    dist.destroy_process_group()
    queue.put((rank, slowest, rate))


def test_two_rank_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=10) for _ in range(2))
    for _, slowest, rate in results:
        assert slowest == 55.0
        assert abs(rate - 2 * 256 * 10 / 0.055) < 1e-6


def test_reference_arm_idle_ranks_exit_cleanly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    run = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert run.returncode == 0
    assert run.stdout.strip() == ""
