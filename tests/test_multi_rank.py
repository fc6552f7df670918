"""The N-rank form of bench.py on the CPU: each rank runs its own replica set
(the path shards by replicas, with no data exchange between ranks), and the
job's throughput is every rank's updates over the slowest rank's time.  Two
gloo ranks on 127.0.0.1, as torchrun would start them."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_local = [0.5, 0.8][rank]  # rank 1 is the slow one
        value, t = bench.job_throughput(t_local, 1000.0, world, True, "cpu")
        out[rank] = (value, t)
    finally:
        torch.distributed.destroy_process_group()


def test_job_throughput_takes_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        value, t = res[rank]
        assert t == pytest.approx(0.8)
        assert value == pytest.approx(2 * 1000.0 / 0.8)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.job_throughput(0.5, 1000.0, 1, False, "cpu") == (2000.0, 0.5)
