"""The N-GPU bench path on the CPU: two gloo ranks (replicas) reduce their
per-frame times with the same helper bench.py uses and rank 0 reports the
whole-job rate from the slowest rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        # rank r's frames took 2 + r ms (plain), 1.5 + 0.25 r (mixed); e2e only on rank 1
        got = bench.reduce_max([2.0 + rank, 1.5 + 0.25 * rank, 3.0 if rank == 1 else 0.0], "cpu")
        out[rank] = (got, bench.replica_rate(got[0], world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        got, rate = res[rank]
        assert got == [3.0, 1.75, 3.0]
        assert rate == pytest.approx(2 * 1e3 / 3.0)
