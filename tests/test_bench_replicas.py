"""The multi-GPU path of bench.py is replicas only: every rank runs its own discharge and the
job value is all ranks' particle-steps over the slowest rank's time.  The aggregation runs here
as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    parts = [1.0e9, 3.0e9][rank]
    secs = [0.5, 2.0][rank]
    out[rank] = bench.aggregate(parts, secs, ws)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ws, port = 2, _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, join=True, start_method="spawn")
    # (1e9 + 3e9) particle-steps over the slowest rank's 2 s
    assert out[0] == pytest.approx(2.0e9) and out[1] == pytest.approx(2.0e9)
