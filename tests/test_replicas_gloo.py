"""The multi-rank bench path (replicas only) with two gloo ranks on the CPU:
every rank gets the slowest rank's timed span from the MAX all-reduce, the
replicas are distinct seeded systems, and the whole-job value counts every
replica."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.5 + rank, "cpu")  # rank 1 took longer
        dist.barrier()
        q.put((rank, slowest, bench.replica_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_the_slowest_span_and_run_distinct_replicas():
    torch = pytest.importorskip("torch")
    import bench
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.5, 2.5]            # both ranks see the slowest span
    assert out[0][2] != out[1][2]                       # distinct seeded replicas
    assert bench.max_over_ranks(3.0, "cpu") == 3.0      # no process group: the value itself
    v1 = bench.aggregate_ns_per_day(1, 1000, 2.5)
    assert bench.aggregate_ns_per_day(2, 1000, 2.5) == pytest.approx(2 * v1)
