"""bench.py with N GPUs runs one independent replica per rank (scenes do not exchange data):
the job time is the max over ranks and the work the sum.  Checked with world_size 2 on gloo."""

import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, units = bench.reduce_over_ranks(10.0 * (rank + 1), 1000.0 * (rank + 1), "cpu")
    q.put((rank, ms, units))
    dist.destroy_process_group()


def test_replica_aggregation_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[1] for o in out] == [20.0, 20.0]
    assert [o[2] for o in out] == [3000.0, 3000.0]
