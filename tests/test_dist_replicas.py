"""The multi-GPU path is replicas only: each rank steps its own copy of the
workload, and bench.py reports the whole job's throughput over the slowest
rank's time.  This checks that host logic with two gloo ranks on the CPU:
the barrier, the max over ranks and the whole-job aggregation."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        ms = [3.0, 5.0][rank]  # rank 1 is the slower replica
        slowest = bench.max_over_ranks(ms, world)
        value = bench.whole_job_gint_per_s(1.0e9, slowest, world)
        out.put((rank, slowest, value))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_replicas_max_over_ranks_and_whole_job_value():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, slowest, value in got:
        assert slowest == 5.0  # every rank sees the slowest replica's time
        assert value == pytest.approx(2 * 1.0e9 / 5e-3 / 1e9)  # both ranks' interactions over that time
