"""The N-GPU form of bench.py runs one replica per rank with no data exchange; its whole-job figures
come from replica_totals (max over ranks of the device and wall times). Checked here with two gloo
ranks on the CPU, each reporting a different time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dev_s = [1.5, 2.0][rank]
    wall_s = [2.5, 2.25][rank]
    out[rank] = bench.replica_totals(100_000, 4, dev_s, wall_s, world, torch.device("cpu"))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            value, dev_s, wall_s = out[r]
            assert dev_s == 2.0 and wall_s == 2.5          # slowest rank on both clocks
            assert value == 2 * 100_000 * 4 / 2.0          # all ranks' edges / the job's time


def test_replica_totals_single_rank():
    import bench
    value, dev_s, wall_s = bench.replica_totals(10, 3, 0.5, 0.75, 1, torch.device("cpu"))
    assert (value, dev_s, wall_s) == (60.0, 0.5, 0.75)
