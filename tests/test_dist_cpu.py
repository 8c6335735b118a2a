"""The multi-process logic of bench.py on CPU: two gloo ranks use the same
helpers the GPU run uses under torchrun (rendezvous on 127.0.0.1, barrier,
max-over-ranks time, whole-job aggregation of replicas), and a non-zero rank
of the reference arm exits without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    ws, r, local = bench.dist_init("gloo")
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier()
    # each replica "took" a different time; the job's time is the slowest
    t = 1.0 + rank
    tmax = bench.reduce_max(t)
    value = bench.aggregate(100.0, ws, tmax)
    bench.barrier()
    dist.destroy_process_group()
    out_q.put((rank, tmax, value))


def test_two_gloo_ranks_aggregate_like_the_gpu_run():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, tmax, value in res:
        assert tmax == 2.0              # max over ranks
        assert value == 100.0 * 2 / 2.0  # all ranks' units / slowest rank's time


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_single_process_helpers_are_identities():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5) == 3.5
    bench.barrier()
    assert bench.aggregate(10.0, 1, 2.0) == 5.0
