"""Chain sharding across ranks (altar/altar/bayesian/MPIAnnealing.py:106-269), host logic on
CPU with two gloo ranks.

ChainShards (the exchange the GPU path uses with NCCL) drives the oracle CATMIP loop split
over two ranks: each rank walks its block of chains with the random streams of their global
indices, the blocks and the accept counters are exchanged after every walk, and the cool
phase runs on the whole population.  Every stage's β and resampling and the final population
equal the single-process run's bit for bit.
"""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from oracle import catmip


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    g = np.linspace(-15e3, 15e3, 16)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    truth = np.array([[1e3, -2e3, 3e3, 2e6]])
    d = catmip.mogi_los(truth, X, Y, los, 0.25, log_strength=False)[0] + \
        np.random.default_rng(7).normal(0, 5e-3, X.size)
    lo, hi = np.array([-1e4, -1e4, 1e3, 1e5]), np.array([1e4, 1e4, 8e3, 1e7])

    def llk(th):
        u = catmip.mogi_los(th, X, Y, los, 0.25, log_strength=False)
        return catmip.diag_llk(u, d, np.full(X.size, 2.5e-5))[0], np.zeros(th.shape[0], bool)

    return llk, lo, hi


def _run(shards=None):
    llk, lo, hi = _problem()
    return catmip.Annealing(llk, lo, hi, chains=512, steps=3, seed=11).run(shards=shards)


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from altar_gb300.bayesian.sharding import ChainShards
    shards = ChainShards(dist)
    assert shards.bounds(512) == (rank * 256, 256)
    r = _run(shards)
    out[rank] = (r["theta"].tobytes(), r["data"].tobytes(), [(s["beta"], s["accepted"], s["rejected"],
                                                             s["unlikely"], s["scaling"]) for s in r["stages"]])
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_run_equals_single_process():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    ref = _run()
    want = (ref["theta"].tobytes(), ref["data"].tobytes(),
            [(s["beta"], s["accepted"], s["rejected"], s["unlikely"], s["scaling"]) for s in ref["stages"]])
    assert len(ref["stages"]) >= 5 and ref["beta"] == 1.0
    for rank in range(world):
        got = out[rank]
        assert got[2] == want[2], rank          # β, acceptance counts and scaling of every stage
        assert got[0] == want[0] and got[1] == want[1], rank


def test_uneven_split_is_rejected():
    class _D:
        @staticmethod
        def get_rank(group=None):
            return 1

        @staticmethod
        def get_world_size(group=None):
            return 3

    from altar_gb300.bayesian.sharding import ChainShards
    s = ChainShards(_D)
    assert s.bounds(300) == (100, 100)
    try:
        s.bounds(301)
    except ValueError:
        return
    raise AssertionError("an uneven split must be rejected")
