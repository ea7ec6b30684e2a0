"""CPU: the bench's multi-GPU path (replicas, no exchange step) with two gloo
ranks: every rank's step time is reduced with MAX and the whole-job value
counts every rank's pixels over that time; the reference arm runs on rank 0
only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, results):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        step = 10.0 + 5.0 * rank           # rank 1 is the slow one
        slowest = bench.max_over_ranks(step, "cpu")
        results[rank] = (slowest, bench.whole_job_gpix(world, 1e9, slowest), bench.dist_info())
    finally:
        dist.destroy_process_group()


def test_two_rank_max_and_whole_job_value():
    port = _free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_rank, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    for rank in (0, 1):
        slowest, value, info = got[rank]
        assert slowest == 15.0
        assert value == pytest.approx(2 * 1e9 / 15e-3 / 1e9)
        assert info == (2, rank, rank)


def test_reference_arm_other_ranks_exit(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        pass
    bench.run_reference(Args())             # rank 1: no work, no output
    assert capsys.readouterr().out == ""
