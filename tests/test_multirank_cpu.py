"""Replicas across ranks (bench.py --gpus N): the host-side reduction of the timings and
simulated time over world_size 2 with the gloo backend on CPU.  No GPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    d = bench.Dist(world)
    d.barrier()
    # each replica advanced its own cloud: times differ, simulated time adds up
    t = d.max(10.0 + rank)
    s = d.sum(1.5 * (rank + 1))
    out.put((rank, t, s))
    d.close()


def test_replica_reductions():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, s in res:
        assert t == 11.0          # slowest replica sets the wall time
        assert s == 1.5 + 3.0     # whole-job simulated time is the sum over replicas
