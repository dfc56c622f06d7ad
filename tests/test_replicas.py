"""Multi-GPU is replicas only (queries are independent): each rank runs its
own index and query stream and the whole-job throughput is the units all
ranks processed over the slowest rank's time.  The aggregation runs here on
CPU ranks (gloo, world size 2), as bench.py runs it over NCCL."""
import os
import socket
import sys

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    v = bench.replicas_throughput(times[rank], world, 1000)
    out[rank] = v
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replica_throughput_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    times = [0.5, 2.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    # 2 ranks x 1000 units over the slower rank's 2.0 s, on every rank
    assert out[0] == out[1] == 1000.0

