"""The N > 1 form of bench.py (independent replicas, one GPU each; the solve does
not shard): two gloo ranks on the CPU check the whole-job aggregation -- the
timed seconds are the maximum over ranks, and throughput counts the units of
all ranks -- that the NCCL run uses."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        t, v = bench.job_throughput(1.0 + rank, 100.0, "cpu")
        q.put((rank, t, v))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_is_max_time_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t, v in res:
        assert t == 2.0 and v == 2 * 100.0 / 2.0


def test_single_process_throughput():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(4.0, 10.0) == (4.0, 2.5)
