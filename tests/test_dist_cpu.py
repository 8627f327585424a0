"""Multi-process host logic of the benchmark on CPU (gloo, two ranks).

The whole-job time of a multi-GPU run is the slowest rank's, reduced with an
all-reduce MAX (the chain exchange itself is tested in test_sharding_cpu.py).
"""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(0.5 + rank, dist)
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert dict(out) == {0: 1.5, 1: 1.5}


def test_single_process_passthrough():
    import bench
    assert bench.max_over_ranks(2.25, None) == 2.25
