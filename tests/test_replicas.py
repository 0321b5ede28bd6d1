"""The multi-GPU path of bench.py is replicas only: each rank runs its own
workload; ranks meet at a barrier and the job rate is all ranks' units over
the slowest rank's time.  Checked here with world_size 2 on the gloo backend
(no GPU): the aggregation and the max-over-ranks reduction."""
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
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    r, w, _ = bench.dist_init("gloo")
    bench.barrier(w)
    seconds = 1.0 + r          # rank 1 is the slow one
    rate, t = bench.replica_throughput(100.0, seconds, w)
    out[r] = (rate, t)
    bench.barrier(w)
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ws, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
        res = dict(out)
    for r in range(ws):
        rate, t = res[r]
        assert t == pytest.approx(2.0)           # the slowest rank's time on every rank
        assert rate == pytest.approx(100.0 * ws / 2.0)
