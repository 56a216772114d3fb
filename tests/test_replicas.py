"""Replicas on several GPUs: bench.py's whole-job figures over ranks (the
slowest rank's time, the sum of collisions), run as two gloo ranks on CPU.
The path has no data-path collective; these two numbers are all that cross
ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    secs, coll = bench.combine_replicas(dist, 1.0 + rank, 1000 * (rank + 1), "cpu")
    out[rank] = (secs, coll)
    dist.barrier()
    dist.destroy_process_group()


def test_combine_replicas_two_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 3000.0)


def test_single_rank_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_replicas(None, 1.5, 42, "cpu") == (1.5, 42.0)
