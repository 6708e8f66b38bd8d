"""The multi-GPU path of bench.py is N independent replicas (the step does not shard within
one process's GPU): each rank times its own steps, the job time is the maximum over ranks, and
the value counts every rank's cells.  Checked here with two gloo ranks on the CPU; the
reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms = 10.0 * (rank + 1)                 # rank 1 is the slow one
        value, t_max = bench.replica_value(ms, ws, cells=1000, steps=5, pg=dist, device="cpu")
        out[rank] = (value, t_max, bench.dist_env())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_value_takes_the_slowest_rank_and_sums_the_cells():
    ws, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for rank in range(ws):
        value, t_max, env = res[rank]
        assert t_max == 20.0
        assert value == pytest.approx(ws * 1000 * 5 / 0.020 / 1e6)
        assert env == (ws, rank, rank)


def test_single_process_value_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_value(8.0, 1, 4000, 4) == (1 * 4000 * 4 / 0.008 / 1e6, 8.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.reference_arm(None, 1000) is None     # returns before reading its arguments
    assert capsys.readouterr().out == ""
