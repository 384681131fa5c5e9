"""The multi-GPU form of bench.py is independent replicas: each rank solves
its own problem, the job time is the slowest rank's and the whole-job rate is
the sum. This checks that bookkeeping with two gloo ranks on the CPU."""
import os
import socket
import sys

import torch.distributed as dist
import torch.multiprocessing as mp

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
    t = 1.0 + rank                       # rank 1 is the slow one
    tm = bench.max_over_ranks(t, world, "cpu")
    out[rank] = (tm, bench.job_rate(world, 10, tm))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == (2.0, 10.0)   # 2 ranks x 10 steps / 2 s
