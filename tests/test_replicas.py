"""Multi-GPU mode is replicas only: every rank runs its own copy of the
workload, with no collective on the data path; the bench takes the slowest
rank's time and sums the node updates.  The aggregation runs here on two
CPU ranks over gloo."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(dist, times[rank], "cpu")
    out.put((rank, t, bench.replica_value(world, 1000, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.002, 0.003]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == pytest.approx(0.003)          # slowest replica
        assert v == pytest.approx(2 * 1000 / 0.003 / 1e6)


def test_reference_arm_only_rank0_works(monkeypatch):
    import argparse
    import bench
    args = argparse.Namespace(steps=1, warmup=0, gpus=2, nx=16, ny=8, nz=8, platelets=1, fibrin=0, seed=2)
    assert bench.run_reference(args, rank=1) == 0
