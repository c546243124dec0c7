"""The multi-GPU mode of bench.py is replicas (one independent solve per rank, no exchange on the data path; the
ranks meet only in a barrier before/after the timed region and a max over ranks of the time). Its host logic runs
here as two gloo ranks on the CPU: process-group setup from the torchrun environment, barrier, max over ranks."""
import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_init(argparse.Namespace(impl="reference"))
    bench.barrier(w)
    m = bench.allmax(w, 1.5 + r)          # each rank's "time"; all must see the slowest
    bench.barrier(w)
    q.put((r, w, local, m, dist.get_backend()))
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[3] == 2.5 and o[4] == "gloo" for o in out)
    assert [o[2] for o in out] == [0, 1]
